// Gate-pass kernels of the sparse statevector engine (sm_103a).
//
// A gate pass updates the table in place; it walks the list of live buckets.
//  * stream pass: a run of gates that never pair keys across 16-key groups -- diagonal gates
//    on any qubit and any gate on qubits 0..3 (the partner sits in the same bucket and is
//    reached with a warp shuffle). A consumer half-warp holds two buckets (lane j holds slot
//    j of both).
//  * pair pass: a gate whose partner key lives in another group (branching gate on a qubit
//    >= 4, or X/Y on a qubit >= 4 with controls the host could not resolve), followed by a
//    stream run. A consumer half-warp takes the group pair (G0, G1 = G0 | m): lane j holds
//    slot j of both groups, so the pair update is lane-local. The group with stored target
//    bit 0 owns the pair; the other owns it only when its partner group is absent -- the
//    reference's pair rule (emulator/device/device_table_FC.cuh:62-110) lifted from keys to
//    16-key groups, which gives the same pairs and the same per-key results. A resolve
//    kernel settles ownership for every list entry before the pass.
// Data movement: every warp prefetches the buckets of its next slots into its own ring of
// shared-memory slots with cp.async (16-byte copies, one commit group per slot), so several
// slots are in flight while it computes; it moves the current slot into registers, applies
// the gates and writes the results back in place with ordinary stores. Every
// pair with at least one present member is read once and written once. A group that appears
// for the first time is claimed with a 128-bit CAS and appended to the list (such groups are
// beyond the entries the pass walks). Pruning follows the reference
// (emulator/device/device_data.cuh:108-156): branching gates drop negligible outputs, swap
// and diagonal gates keep every key.
#include "sqc_kernels.h"
#include "sqc_pass_dev.cuh"

#include <algorithm>

namespace sqc {

namespace {

constexpr unsigned long long kDirectMaxBuckets = 1ULL << 20;   // larger tables take staged passes

// Block-reduce the pass counters; the last block to finish publishes the pass (key count,
// list length, empty buckets, pass counter, amp updates, algorithmic bytes). Nothing is
// published when a pass failed.
__device__ void finish_pass(Ctl* ctl, unsigned long long n, unsigned long long e, unsigned long long u,
                            unsigned long long nnz_in, bool keys_fixed, bool pair, unsigned amp_bytes) {
    __shared__ unsigned long long red[3][32];
    __shared__ bool last;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    n = warp_sum(n); e = warp_sum(e); u = warp_sum(u);
    if (lane == 0) { red[0][w] = n; red[1][w] = e; red[2][w] = u; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bn = 0, be = 0, bu = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { bn += red[0][i]; be += red[1][i]; bu += red[2][i]; }
        if (bn) atomicAdd(&ctl->acc_nnz, bn);
        if (be) atomicAdd(&ctl->acc_empty, be);
        if (bu) atomicAdd(&ctl->acc_upd, bu);
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->done, 1u);
        last = prev == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const unsigned long long tn = atomicExch(&ctl->acc_nnz, 0ULL);
        const unsigned long long te = atomicExch(&ctl->acc_empty, 0ULL);
        const unsigned long long tu = atomicExch(&ctl->acc_upd, 0ULL);
        if (*(volatile unsigned int*)&ctl->status == 0) {
            ctl->nnz = tn;
            ctl->empty_groups = te;
            ctl->list_n = *(volatile unsigned long long*)&ctl->list_tail;
            ctl->amp_updates += tu;
            const unsigned long long ab = keys_fixed ? nnz_in * (8ULL + 2ULL * amp_bytes) : (nnz_in + tn) * (8ULL + amp_bytes);
            ctl->alg_bytes += ab;
            if (pair) ctl->alg_bytes_pair += ab;
            ctl->seq += 1;
        }
        ctl->done = 0;
        ctl->work = 0;
        ctl->units_n = 0;
        __threadfence();
    }
}

// ---- direct pass (tables up to kDirectMaxBuckets) ------------------------------------------
// For small states the extra launch and the pipeline fill of a staged pass cost more than
// they save: each warp takes four list entries at a time, settles ownership inline (four
// lookups in parallel), packs owned pairs two per warp and loads its slots straight into
// registers.
// True when a pass with nx cross-group qubits could leave more groups than the table takes.
__device__ __forceinline__ bool could_overflow(const PassArgs& a, unsigned long long n) {
    const unsigned long long grown = umin64(a.grow_bound, n << a.nx);
    return grown > a.max_groups;
}

// Blocks per SM the direct kernel's registers are sized for: FP32 fits four without spills,
// FP64 three.
// Passes read their gates from shared memory, staged once per block (FP64: 2-3% faster on large
// tables; FP32 staged passes 0.6% on the 64-qubit workload since the per-slot bucket index
// became 32 bits: before, the staging's registers cost FP32 more than it saved). Blocks per SM
// the staged kernel's registers are sized for: FP64 six; FP32 left to the compiler (0: no
// minimum; seven measured no better).
template <class T, int NX> struct StagedOcc {
    static constexpr int kMin = sizeof(T) == 8 ? (NX == 3 ? 4 : 6) : 0;   // FP64 octets: 53 KB rings, four blocks
};
template <class T> struct StageGates { static constexpr bool kOn = true; };
// The direct kernel's FP32 octet passes gain from it too (1.7% on the 40-qubit workload).
template <class T, int NX> struct DirectStage { static constexpr bool kOn = sizeof(T) == 8 || NX == 3; };

// Octet passes (three cross-group qubits) hold four slots per lane: FP64 two blocks, FP32 three.
template <class T, int NX> struct DirectOcc {
    static constexpr int kMin = NX == 3 ? (sizeof(T) == 8 ? 2 : 3) : (sizeof(T) == 8 ? 3 : 4);
};

// The work of one direct pass: warps take four list entries at a time through next4 (a value
// >= n ends the pass), so they finish together whatever the number of units each group of
// entries owns. With SMEM the gates are read from shared memory (sg[i] = gate g0 + i), else
// through L1. Counters accumulate per thread.
template <class T, int NX, bool SMEM, class Next>
__device__ __forceinline__ void direct_work(const PassArgs& a, const SmemGate* sg, unsigned ep, unsigned long long n,
                                            Next&& next4, unsigned long long& cnt_nnz, unsigned long long& cnt_empty,
                                            unsigned long long& upd) {
    Ctl* ctl = a.ctl;
    const TableDev t = a.t;
    const int lane = threadIdx.x & 31, half = lane >> 4, j = lane & 15;
    Val<T> va, vb;
    if constexpr (NX == 0) {
        for (unsigned long long e0 = next4(); e0 < n; e0 = next4()) {
            const unsigned long long ea = e0 + 2 * half, eb = ea + 1;
            const long long ba = ea < n ? (long long)t.list[ea] : -1;
            const long long bb = eb < n ? (long long)t.list[eb] : -1;
            const unsigned long long Ga = ba >= 0 ? load_hdr(t.hdr + ba).group : 0ULL;
            const unsigned long long Gb = bb >= 0 ? load_hdr(t.hdr + bb).group : 0ULL;
            load_val_g<T>(t, va, Ga, ba, j);
            load_val_g<T>(t, vb, Gb, bb, j);
            if constexpr (SMEM) run_gates_s<T>(sg, a.gates, a.g0, a.g1, va, vb, lane, a.prune, upd);
            else run_gates<T>(a.gates, a.g0, a.g1, va, vb, lane, a.prune, upd);
            write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
            write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
        }
    } else if constexpr (NX == 3) {
        const unsigned long long m1 = 1ULL << (a.q1 - kSlotBits);
        const unsigned long long m2 = 1ULL << (a.q2 - kSlotBits);
        const unsigned long long m3 = 1ULL << (a.q3 - kSlotBits);
        for (unsigned long long e0 = next4(); e0 < n; e0 = next4()) {
            long long mb;
            unsigned long long G0;
            const unsigned om = units4<3>(t, ep, e0, n, m1, m2, lane, &mb, &G0, m3);
            run_units8<T, SMEM>(t, ep, ctl, a.gates, sg, a.g0, a.g1, m1, m2, m3, om, mb, G0, lane, a.prune, cnt_nnz,
                                cnt_empty, upd);
        }
    } else {
        const unsigned long long m1 = 1ULL << (a.q1 - kSlotBits);
        const unsigned long long m2 = NX == 2 ? 1ULL << (a.q2 - kSlotBits) : 0ULL;
        for (unsigned long long e0 = next4(); e0 < n; e0 = next4()) {
            long long mb;
            unsigned long long G0;
            const unsigned om = units4<NX>(t, ep, e0, n, m1, m2, lane, &mb, &G0);
            run_units4<T, NX, true, SMEM>(t, ep, ctl, a.gates, sg, a.g0, a.g1, m1, m2, om, mb, G0, lane, a.prune, va,
                                          vb, cnt_nnz, cnt_empty, upd);
        }
    }
}

template <class T, int NX>
__global__ void __launch_bounds__(kThreads, DirectOcc<T, NX>::kMin) direct_kernel(PassArgs a) {
    constexpr bool kSmem = NX == 3 ? DirectStage<T, NX>::kOn : StageGates<T>::kOn;
    __shared__ SmemGate sg[kSmem ? kMaxRun : 1];
    // the gates were copied to the device before the first pass of their flush started, and
    // no kernel writes them: they are staged while the previous pass drains
    if constexpr (kSmem) stage_gates(sg, a.gates, a.g0, a.g1);
    wait_prior_grid();
    allow_next_grid();
    Ctl* ctl = a.ctl;
    if (*(volatile unsigned int*)&ctl->status) return;
    const unsigned long long n = ctl->list_n;
    if (NX > 0 && could_overflow(a, n)) {   // refuse before touching the state
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctl->status, 0u, (unsigned)ST_GROW);
        return;
    }
    const unsigned ep = ctl->epoch;
    const unsigned long long nnz_in = ctl->nnz;
    const int lane = threadIdx.x & 31;
    unsigned long long cnt_nnz = 0, cnt_empty = 0, upd = 0;
    auto next4 = [&]() -> unsigned long long {
        unsigned long long e = 0;
        if (lane == 0) e = atomicAdd(&ctl->work, 4ULL);
        return shfl64(e, 0);
    };
    direct_work<T, NX, kSmem>(a, sg, ep, n, next4, cnt_nnz, cnt_empty, upd);
    finish_pass(ctl, cnt_nnz, cnt_empty, upd, nnz_in, a.keys_fixed != 0, NX > 0, a.amp_bytes);
}

// ---- tiny states: every pass of a flush in one single-block launch --------------------------
// For tables of at most kTinyMaxBuckets buckets a pass is a few microseconds of dependent
// loads, and separate launches would cost more than the work. One block runs the passes in
// order: the pass's gates are staged in shared memory, warps claim list entries from a
// shared-memory counter, the block reduces and publishes the pass (as finish_pass does) and
// synchronises before the next. A pass that could overflow the table refuses as a direct pass
// does, and the passes after it do not run; the host repairs and replays from there.
template <class T>
__global__ void __launch_bounds__(kThreads) tiny_kernel(PassArgs a, const TinyPass* __restrict__ tp, uint32_t np) {
    __shared__ SmemGate sg[kMaxRun];
    __shared__ unsigned long long claim_sh;
    __shared__ unsigned long long red[3][kThreads / 32];
    __shared__ int stop;
    Ctl* ctl = a.ctl;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t p = 0; p < np; ++p) {
        if (threadIdx.x == 0) {
            stop = *(volatile unsigned int*)&ctl->status != 0;
            claim_sh = 0;
        }
        __syncthreads();
        if (stop) return;
        PassArgs b = a;
        const TinyPass q = tp[p];
        b.g0 = q.g0;
        b.g1 = q.g1;
        b.nx = q.nx;
        b.q1 = q.q1;
        b.q2 = q.q2;
        b.q3 = q.q3;
        b.keys_fixed = q.keys_fixed;
        b.grow_bound = q.grow_bound;
        const unsigned long long n = *(volatile unsigned long long*)&ctl->list_n;
        if (b.nx > 0 && could_overflow(b, n)) {   // refuse before touching the state
            if (threadIdx.x == 0) atomicCAS(&ctl->status, 0u, (unsigned)ST_GROW);
            return;
        }
        stage_gates(sg, b.gates, b.g0, b.g1);
        const unsigned ep = *(volatile unsigned int*)&ctl->epoch;
        const unsigned long long nnz_in = *(volatile unsigned long long*)&ctl->nnz;
        unsigned long long cnt_nnz = 0, cnt_empty = 0, upd = 0;
        auto next4 = [&]() -> unsigned long long {
            unsigned long long e = 0;
            if (lane == 0) e = atomicAdd(&claim_sh, 4ULL);
            return shfl64(e, 0);
        };
        switch (b.nx) {
        case 0: direct_work<T, 0, true>(b, sg, ep, n, next4, cnt_nnz, cnt_empty, upd); break;
        case 1: direct_work<T, 1, true>(b, sg, ep, n, next4, cnt_nnz, cnt_empty, upd); break;
        case 2: direct_work<T, 2, true>(b, sg, ep, n, next4, cnt_nnz, cnt_empty, upd); break;
        default: direct_work<T, 3, true>(b, sg, ep, n, next4, cnt_nnz, cnt_empty, upd); break;
        }
        cnt_nnz = warp_sum(cnt_nnz);
        cnt_empty = warp_sum(cnt_empty);
        upd = warp_sum(upd);
        if (lane == 0) { red[0][w] = cnt_nnz; red[1][w] = cnt_empty; red[2][w] = upd; }
        __syncthreads();
        if (threadIdx.x == 0 && *(volatile unsigned int*)&ctl->status == 0) {
            unsigned long long tn = 0, te = 0, tu = 0;
            for (int i = 0; i < kThreads / 32; ++i) { tn += red[0][i]; te += red[1][i]; tu += red[2][i]; }
            ctl->nnz = tn;
            ctl->empty_groups = te;
            ctl->list_n = *(volatile unsigned long long*)&ctl->list_tail;
            ctl->amp_updates += tu;
            const unsigned long long ab = b.keys_fixed ? nnz_in * (8ULL + 2ULL * b.amp_bytes)
                                                       : (nnz_in + tn) * (8ULL + b.amp_bytes);
            ctl->alg_bytes += ab;
            if (b.nx > 0) ctl->alg_bytes_pair += ab;
            ctl->seq += 1;
        }
        __syncthreads();   // the pass is published before the next one reads it
    }
}

constexpr int kResolveThreads = 256;

// ---- resolve: the owned units of a pass that pairs groups, before the pass -----------------
// Two phases per chunk of kResolveThreads list entries:
//  * ownership: every thread takes one entry and looks up the unit's members of smaller index
//    (the entry owns its unit iff none is live; usually one lookup settles it). Each block
//    reserves room for its owned units with one atomic on ctl->units_n and places them
//    densely, in no particular order;
//  * members: the owners' remaining lookups are spread over the warp's lanes, K = 2^nx lanes
//    per owner (lane k looks up member k), 32 / K owners at a time, so an owner's members are
//    found in one round trip rather than one after another.
// The staged pass deals the units out evenly.
template <int NX>
__global__ void __launch_bounds__(kResolveThreads) resolve_kernel(PassArgs a) {
    constexpr int K = 1 << NX;
    __shared__ unsigned warp_at[2][kResolveThreads / 32];   // two sets: chunk parity
    __shared__ unsigned long long base_sh[2];
    Ctl* ctl = a.ctl;
    if (*(volatile unsigned int*)&ctl->status) return;
    const unsigned long long n = ctl->list_n;
    if (could_overflow(a, n)) {   // refuse before touching the state
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctl->status, 0u, (unsigned)ST_GROW);
        return;
    }
    const unsigned ep = ctl->epoch;
    const unsigned long long m1 = 1ULL << (a.q1 - kSlotBits);
    const unsigned long long m2 = NX >= 2 ? 1ULL << (a.q2 - kSlotBits) : 0ULL;
    const unsigned long long m3 = NX == 3 ? 1ULL << (a.q3 - kSlotBits) : 0ULL;
    auto member = [&](unsigned long long G0, int k) {
        return G0 | ((k & 1) ? m1 : 0ULL) | ((k & 2) ? m2 : 0ULL) | ((k & 4) ? m3 : 0ULL);
    };
    const TableDev t = a.t;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int par = 0;
    for (unsigned long long c0 = (unsigned long long)blockIdx.x * kResolveThreads; c0 < n;
         c0 += (unsigned long long)gridDim.x * kResolveThreads, par ^= 1) {
        const unsigned long long e = c0 + threadIdx.x;
        bool own = false;
        unsigned b = kNoBucket;
        int idx = 0;
        unsigned long long G0 = 0;
        if (e < n) {
            b = t.list[e];
            const unsigned long long G = load_hdr(t.hdr + b).group;
            idx = ((G & m1) ? 1 : 0) | ((NX >= 2 && (G & m2)) ? 2 : 0) | ((NX == 3 && (G & m3)) ? 4 : 0);
            G0 = G & ~(m1 | m2 | m3);
            own = true;
            for (int k = 0; k < idx && own; ++k) own = lookup_group(t, ep, member(G0, k)) < 0;
        }
        const unsigned bal = __ballot_sync(kFull, own);
        if (lane == 0) warp_at[par][w] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (int i = 0; i < kResolveThreads / 32; ++i) {
                const unsigned c = warp_at[par][i];
                warp_at[par][i] = tot;
                tot += c;
            }
            base_sh[par] = tot ? atomicAdd(&ctl->units_n, (unsigned long long)tot) : 0ULL;
        }
        __syncthreads();
        const unsigned long long pos = base_sh[par] + warp_at[par][w] + __popc(bal & ((1u << lane) - 1u));
        // members of this warp's owners, 32 / K owners per round, lane r * K + k on member k
        unsigned rem = bal;
        while (rem) {
            int src = -1;
#pragma unroll
            for (int r = 0; r < 32 / K; ++r) {
                const int o = rem ? __ffs(rem) - 1 : -1;
                if (rem) rem &= rem - 1;
                if (r == lane / K) src = o;
            }
            const int k = lane % K;
            const unsigned long long sG0 = shfl64(G0, src < 0 ? 0 : src);
            const int sidx = __shfl_sync(kFull, idx, src < 0 ? 0 : src);
            const unsigned sb = __shfl_sync(kFull, b, src < 0 ? 0 : src);
            const unsigned long long spos = shfl64(pos, src < 0 ? 0 : src);
            if (src >= 0) {
                // members below the owner's index are absent (that is what made it the owner)
                const long long mb = k == sidx ? (long long)sb : k < sidx ? -1LL : lookup_group(t, ep, member(sG0, k));
                Unit* u = t.units + spos;
                u->b[k] = mb < 0 ? kNoBucket : (unsigned)mb;
                if (k == 0) u->G0 = sG0;
            }
        }
        // the next chunk uses the other set of warp_at / base_sh, and the chunk after it writes
        // this set again only past the next chunk's barriers, which no warp passes before it
        // has read this set (one barrier fewer per chunk than a barrier here: FP64 64-qubit
        // workload 74.09 -> 73.68 ms, FP32 28.23 -> 28.11 ms)
    }
}

// ---- staged pass -------------------------------------------------------------------------
// Every warp is a worker with its own ring of D = RingDepth shared-memory slots. It copies the
// buckets of the slot D-1 steps ahead with cp.async (one commit group per slot), waits
// for the current slot's group, moves the slot into registers, applies the gates and writes
// back in place. A slot holds the buckets of one item: four list entries (stream pass), two
// owned pairs (pair pass), one owned quad, or one owned octet (eight buckets).
constexpr int kWarpsPerBlock = 4;
constexpr int kStagedThreads = 32 * kWarpsPerBlock;
// FP32 octet rings hold three slots (two items in flight, 27 KB per block): the same six
// blocks per SM as four (registers bound them), with more of the SM's memory left to L1
// (64-qubit FP32 workload 0.6% faster). Forcing seven or eight blocks spills registers (7-16%
// slower).
template <class T, int NX> struct RingDepth { static constexpr int k = (sizeof(T) == 4 && NX == 3) ? 3 : 4; };

// A ring slot: the buckets of one item, NB = 4 (stream, pair and quad passes) or 8 (octets).
template <class T, int NB> struct Slot {
    unsigned long long keys[NB][kSlots];
    typename AmpT<T>::V amps[NB][kSlots];
    Header hdr[NB];             // stream passes: copied headers (groups)
    unsigned long long G[NB];   // pair passes: group of each held bucket
    unsigned int b[NB];         // bucket index, kNoBucket when absent
    int n;                      // 0: nothing more for this warp
    int pad[3];
};
template <int NX> struct SlotBuckets { static constexpr int kN = NX == 3 ? 8 : 4; };

template <class T, int NB>
__device__ __forceinline__ void load_val_s(Val<T>& v, unsigned long long G, unsigned b, const Slot<T, NB>& sl, int k,
                                           int j) {
    v.key = (G << kSlotBits) | (unsigned long long)j;
    v.b = b == kNoBucket ? -1 : (int)b;
    v.dirty = false;
    v.pres = false;
    v.amp = czero<T>();
    if (b != kNoBucket) {
        v.pres = slot_present(sl.keys[k][j], j);
        if (v.pres) {
            const typename AmpT<T>::V x = sl.amps[k][j];
            v.amp = Cx<T>{x.x, x.y};
        }
    }
    v.pres0 = v.pres;
}

// Where a warp's slots come from. The items of a pass -- four list entries (stream pass), two
// owned pairs (pair pass), one owned quad or one owned octet -- are dealt out round robin: warp
// w of W takes items w, w + W, w + 2W, ... Items cost the same, so the warps finish together,
// and every warp knows its next item in advance: the bucket indices of the item after the one
// being issued are loaded one issue ahead (lanes 0..NB-1, one bucket each), so no issue waits
// on them.
struct SlotSource {
    unsigned long long item, stride;   // the next item to load, W
    unsigned long long count;          // items of the pass
    unsigned nb;                       // prefetched bucket of this lane (lanes 0..NB-1)
    unsigned long long ng;             // ... and its group (pair, quad and octet passes)
    bool nany;                         // the prefetched item exists
};

template <int NX>
__device__ __forceinline__ void fetch_item(SlotSource& src, const TableDev& t, unsigned long long n,
                                           unsigned long long units, unsigned long long m1, unsigned long long m2,
                                           unsigned long long m3, int lane) {
    const unsigned long long i = src.item;
    src.item += src.stride;
    src.nany = i < src.count;
    src.nb = kNoBucket;
    src.ng = 0;
    if (!src.nany || lane >= SlotBuckets<NX>::kN) return;
    if (NX == 0) {
        const unsigned long long e = 4 * i + (unsigned long long)lane;
        if (e < n) src.nb = t.list[e];
    } else if (NX == 1) {   // two pairs: buckets (G0, G0|m1) of units 2i and 2i + 1
        const unsigned long long u = 2 * i + (unsigned long long)(lane >> 1);
        if (u < units) {
            const Unit un = t.units[u];
            src.nb = (lane & 1) ? un.b[1] : un.b[0];
            src.ng = (lane & 1) ? (un.G0 | m1) : un.G0;
        }
    } else {                // one quad or octet: bucket k is member k = i0 + 2*i1 + 4*i2
        src.nb = t.units[i].b[lane];
        src.ng = t.units[i].G0 | ((lane & 1) ? m1 : 0ULL) | ((lane & 2) ? m2 : 0ULL) | ((lane & 4) ? m3 : 0ULL);
    }
}

// Copy the prefetched item's buckets into a ring slot (cp.async, one commit group) and
// prefetch the next item.
template <class T, int NX>
__device__ __forceinline__ void issue_slot(Slot<T, SlotBuckets<NX>::kN>& sl, const TableDev& t, SlotSource& src,
                                           unsigned long long n, unsigned long long units, unsigned long long m1,
                                           unsigned long long m2, unsigned long long m3, int lane) {
    constexpr int NB = SlotBuckets<NX>::kN;
    constexpr uint32_t kAmp = (uint32_t)(sizeof(typename AmpT<T>::V) * kSlots);
    constexpr int kKeyChunks = 128 / 16, kAmpChunks = (int)(kAmp / 16);
    constexpr int kChunks = NB * (kKeyChunks + kAmpChunks) + (NX ? 0 : 4);
    const unsigned bk = src.nb;
    const unsigned long long Gk = src.ng;
    const bool any = src.nany;
    fetch_item<NX>(src, t, n, units, m1, m2, m3, lane);
    const unsigned b0 = __shfl_sync(kFull, bk, 0), b1 = __shfl_sync(kFull, bk, 1);
    const unsigned b2 = __shfl_sync(kFull, bk, 2), b3 = __shfl_sync(kFull, bk, 3);
    unsigned b4 = kNoBucket, b5 = kNoBucket, b6 = kNoBucket, b7 = kNoBucket;
    if constexpr (NB == 8) {
        b4 = __shfl_sync(kFull, bk, 4); b5 = __shfl_sync(kFull, bk, 5);
        b6 = __shfl_sync(kFull, bk, 6); b7 = __shfl_sync(kFull, bk, 7);
    }
    if (lane < NB) {
        sl.b[lane] = bk;
        sl.G[lane] = Gk;
    }
    if (lane == 0) sl.n = any ? 1 : 0;
    for (int c = lane; c < kChunks; c += 32) {
        int k, off;
        const char* s;
        char* d;
        if (c < NB * kKeyChunks) {
            k = c / kKeyChunks; off = (c % kKeyChunks) * 16;
        } else if (c < NB * (kKeyChunks + kAmpChunks)) {
            const int x = c - NB * kKeyChunks;
            k = x / kAmpChunks; off = (x % kAmpChunks) * 16;
        } else {
            k = c - NB * (kKeyChunks + kAmpChunks); off = 0;
        }
        const unsigned b = k < 4 ? (k == 0 ? b0 : k == 1 ? b1 : k == 2 ? b2 : b3)
                                 : (k == 4 ? b4 : k == 5 ? b5 : k == 6 ? b6 : b7);
        if (b == kNoBucket) continue;
        if (c < NB * kKeyChunks) {
            s = reinterpret_cast<const char*>(t.keys + (size_t)b * kSlots) + off;
            d = reinterpret_cast<char*>(sl.keys[k]) + off;
        } else if (c < NB * (kKeyChunks + kAmpChunks)) {
            s = reinterpret_cast<const char*>(t.amps) + (size_t)b * kAmp + off;
            d = reinterpret_cast<char*>(sl.amps[k]) + off;
        } else {
            s = reinterpret_cast<const char*>(t.hdr + b);
            d = reinterpret_cast<char*>(&sl.hdr[k]);
        }
        cp_async16(d, s);
    }
    cp_async_commit();
}


template <class T, int NX>
__global__ void __launch_bounds__(kStagedThreads, StagedOcc<T, NX>::kMin) staged_kernel(PassArgs a) {
    constexpr int NB = SlotBuckets<NX>::kN;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int D = RingDepth<T, NX>::k;
    Slot<T, NB>* ring = reinterpret_cast<Slot<T, NB>*>(smem_raw) + (threadIdx.x >> 5) * D;
    __shared__ SmemGate sg[StageGates<T>::kOn ? kMaxRun : 1];

    Ctl* ctl = a.ctl;
    if (*(volatile unsigned int*)&ctl->status) return;
    if constexpr (StageGates<T>::kOn) stage_gates(sg, a.gates, a.g0, a.g1);
    const unsigned long long n = ctl->list_n;
    const unsigned ep = ctl->epoch;
    const unsigned long long nnz_in = ctl->nnz;
    const TableDev t = a.t;
    const int lane = threadIdx.x & 31, half = lane >> 4, jj = lane & 15;
    const unsigned long long m1 = NX ? 1ULL << (a.q1 - kSlotBits) : 0ULL;
    const unsigned long long m2 = NX >= 2 ? 1ULL << (a.q2 - kSlotBits) : 0ULL;
    const unsigned long long m3 = NX == 3 ? 1ULL << (a.q3 - kSlotBits) : 0ULL;
    // owned units, written by this pass's resolve kernel (stream passes: none)
    const unsigned long long units = NX ? umin64(*(volatile unsigned long long*)&ctl->units_n, n) : 0ULL;
    SlotSource src;
    src.item = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    src.stride = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    src.count = NX == 0 ? (n + 3) / 4 : NX == 1 ? (units + 1) / 2 : units;
    fetch_item<NX>(src, t, n, units, m1, m2, m3, lane);
    unsigned long long cnt_nnz = 0, cnt_empty = 0, upd = 0;
    for (int d = 0; d < D - 1; ++d) issue_slot<T, NX>(ring[d], t, src, n, units, m1, m2, m3, lane);
    Val<T> va, vb;
    for (unsigned step = 0;; ++step) {
        issue_slot<T, NX>(ring[(step + D - 1) % D], t, src, n, units, m1, m2, m3, lane);
        cp_async_wait<D - 1>();
        __syncwarp();
        const Slot<T, NB>& sl = ring[step % D];
        if (sl.n == 0) break;
        if constexpr (NX == 3) {   // one octet: this half's members (i0, half, i2), four slots per lane
            const int k0 = 2 * half;
            Val<T> vc, vd;
            load_val_s<T>(va, sl.G[k0], sl.b[k0], sl, k0, jj);
            load_val_s<T>(vb, sl.G[k0 + 1], sl.b[k0 + 1], sl, k0 + 1, jj);
            load_val_s<T>(vc, sl.G[k0 + 4], sl.b[k0 + 4], sl, k0 + 4, jj);
            load_val_s<T>(vd, sl.G[k0 + 5], sl.b[k0 + 5], sl, k0 + 5, jj);
            __syncwarp();
            run_gates4<T, StageGates<T>::kOn>(sg, a.gates, a.g0, a.g1, va, vb, vc, vd, lane, a.prune, upd);
            const long long fa = write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
            const long long fb = write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
            const long long fc = write_val<T>(t, ep, vc, lane, &ctl->status, cnt_nnz, cnt_empty);
            const long long fd = write_val<T>(t, ep, vd, lane, &ctl->status, cnt_nnz, cnt_empty);
            append_new(t, ctl, fa, fb, lane);
            append_new(t, ctl, fc, fd, lane);
            continue;
        }
        const int ka = 2 * half, kb = ka + 1;
        const unsigned ba = sl.b[ka], bb = sl.b[kb];
        unsigned long long Ga, Gb;
        if (NX) {
            Ga = sl.G[ka];
            Gb = sl.G[kb];
        } else {
            Ga = ba != kNoBucket ? sl.hdr[ka].group : 0ULL;
            Gb = bb != kNoBucket ? sl.hdr[kb].group : 0ULL;
        }
        load_val_s<T>(va, Ga, ba, sl, ka, jj);
        load_val_s<T>(vb, Gb, bb, sl, kb, jj);
        __syncwarp();
        if constexpr (StageGates<T>::kOn) run_gates_s<T>(sg, a.gates, a.g0, a.g1, va, vb, lane, a.prune, upd);
        else run_gates<T>(a.gates, a.g0, a.g1, va, vb, lane, a.prune, upd);
        const long long fa = write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
        const long long fb = write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
        if (NX) append_new(t, ctl, fa, fb, lane);
    }
    cp_async_wait<0>();   // nothing may still be landing in shared memory when the block exits
    finish_pass(ctl, cnt_nnz, cnt_empty, upd, nnz_in, a.keys_fixed != 0, NX > 0, a.amp_bytes);
}

template <class T, int NX>
constexpr size_t staged_smem() {
    return (size_t)kWarpsPerBlock * RingDepth<T, NX>::k * sizeof(Slot<T, SlotBuckets<NX>::kN>);
}

template <class K>
int occupancy(K kernel, int threads, size_t smem) {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem);
    return n > 0 ? n : 1;
}

// Resident blocks per SM of each staged-kernel instantiation (queried once per process).
// Occupancy of one staged-kernel instantiation; rings above the 48 KB default (FP64 octets)
// are allowed first.
template <class T, int NX>
int staged_occupancy() {
    if (staged_smem<T, NX>() > (48u << 10))
        cudaFuncSetAttribute(staged_kernel<T, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)staged_smem<T, NX>());
    return occupancy(staged_kernel<T, NX>, kStagedThreads, staged_smem<T, NX>());
}

int staged_residency(bool dbl, int nx) {
    static int cache[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    int& c = cache[dbl ? 1 : 0][nx];
    if (!c) {
        if (dbl) c = nx == 0 ? staged_occupancy<double, 0>() : nx == 1 ? staged_occupancy<double, 1>()
                   : nx == 2 ? staged_occupancy<double, 2>() : staged_occupancy<double, 3>();
        else c = nx == 0 ? staged_occupancy<float, 0>() : nx == 1 ? staged_occupancy<float, 1>()
                 : nx == 2 ? staged_occupancy<float, 2>() : staged_occupancy<float, 3>();
    }
    return c;
}

int direct_residency(bool dbl, int nx) {
    static int cache[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    int& c = cache[dbl ? 1 : 0][nx];
    if (!c) {
        if (dbl) c = nx == 0 ? occupancy(direct_kernel<double, 0>, kThreads, 0)
                   : nx == 1 ? occupancy(direct_kernel<double, 1>, kThreads, 0)
                   : nx == 2 ? occupancy(direct_kernel<double, 2>, kThreads, 0)
                             : occupancy(direct_kernel<double, 3>, kThreads, 0);
        else c = nx == 0 ? occupancy(direct_kernel<float, 0>, kThreads, 0)
                 : nx == 1 ? occupancy(direct_kernel<float, 1>, kThreads, 0)
                 : nx == 2 ? occupancy(direct_kernel<float, 2>, kThreads, 0)
                           : occupancy(direct_kernel<float, 3>, kThreads, 0);
    }
    return c;
}

constexpr unsigned long long kTinyMaxBuckets = 4096;

// Launch a direct pass with programmatic stream serialization: its blocks may be scheduled
// once the previous kernel in the stream has let them (allow_next_grid), and they wait for
// that kernel's completion in wait_prior_grid before touching the state. Direct passes take
// their work from an atomic counter, so blocks placed unevenly while the previous pass drains
// cost nothing. Resolve and staged passes split their work statically over the grid; launched
// this way they measured 20-30% slower on 2^24-key tables, so they keep plain launches.
template <class K>
cudaError_t launch_dep(K kernel, int grid, int threads, size_t smem, const PassArgs& a, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

template <class T, int NX>
cudaError_t launch_direct(const PassArgs& a, int grid, cudaStream_t st) {
    return launch_dep(direct_kernel<T, NX>, grid, kThreads, 0, a, st);
}

template <class T, int NX>
cudaError_t launch_staged(const PassArgs& a, int grid, cudaStream_t st) {
    staged_kernel<T, NX><<<grid, kStagedThreads, staged_smem<T, NX>(), st>>>(a);
    return cudaGetLastError();
}

}  // namespace

bool tiny_table(unsigned long long buckets) { return buckets <= kTinyMaxBuckets; }

int launch_tiny(const PassArgs& a, const TinyPass* passes, uint32_t np, bool dbl, cudaStream_t st) {
    if (a.t.mask + 1 > kTinyMaxBuckets) return -1;
    if (dbl) tiny_kernel<double><<<1, kThreads, 0, st>>>(a, passes, np);
    else tiny_kernel<float><<<1, kThreads, 0, st>>>(a, passes, np);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int launch_pass(const PassArgs& a, unsigned long long list_hint, bool dbl, int sms, cudaStream_t st) {
    // list_hint bounds the live-bucket count; grids are sized from it (one resident wave at
    // most); the kernels read the exact count. Tables of up to kDirectMaxBuckets buckets
    // (states that have never needed more) take the direct pass.
    const int nx = (int)a.nx;
    if (nx < 0 || nx > 3) return -1;
    if (a.t.mask + 1 <= kDirectMaxBuckets) {
        const unsigned long long wave = (unsigned long long)sms * direct_residency(dbl, nx);
        const unsigned long long g = (list_hint / 4 + 1 + kThreads / 32 - 1) / (kThreads / 32);
        const int grid = (int)std::max<unsigned long long>(1, std::min(g, wave));
        cudaError_t e;
        if (dbl) {
            if (nx == 0) e = launch_direct<double, 0>(a, grid, st);
            else if (nx == 1) e = launch_direct<double, 1>(a, grid, st);
            else if (nx == 2) e = launch_direct<double, 2>(a, grid, st);
            else e = launch_direct<double, 3>(a, grid, st);
        } else {
            if (nx == 0) e = launch_direct<float, 0>(a, grid, st);
            else if (nx == 1) e = launch_direct<float, 1>(a, grid, st);
            else if (nx == 2) e = launch_direct<float, 2>(a, grid, st);
            else e = launch_direct<float, 3>(a, grid, st);
        }
        return e == cudaSuccess ? 1 : -1;
    }
    int launched = 0;
    if (nx) {
        const unsigned long long chunks = list_hint / kResolveThreads + 1;
        const int g = (int)std::max<unsigned long long>(1, std::min<unsigned long long>(chunks, (unsigned long long)sms * 8));
        if (nx == 1) resolve_kernel<1><<<g, kResolveThreads, 0, st>>>(a);
        else if (nx == 2) resolve_kernel<2><<<g, kResolveThreads, 0, st>>>(a);
        else resolve_kernel<3><<<g, kResolveThreads, 0, st>>>(a);
        if (cudaGetLastError() != cudaSuccess) return -1;
        ++launched;
    }
    const unsigned long long items = nx >= 2 ? list_hint + 1 : nx == 1 ? list_hint / 2 + 1 : (list_hint + 3) / 4;
    const unsigned long long wave = (unsigned long long)sms * staged_residency(dbl, nx);
    const int grid = (int)std::max<unsigned long long>(1, std::min(wave, (items + 3) / 4));
    cudaError_t e;
    if (dbl) {
        if (nx == 0) e = launch_staged<double, 0>(a, grid, st);
        else if (nx == 1) e = launch_staged<double, 1>(a, grid, st);
        else if (nx == 2) e = launch_staged<double, 2>(a, grid, st);
        else e = launch_staged<double, 3>(a, grid, st);
    } else {
        if (nx == 0) e = launch_staged<float, 0>(a, grid, st);
        else if (nx == 1) e = launch_staged<float, 1>(a, grid, st);
        else if (nx == 2) e = launch_staged<float, 2>(a, grid, st);
        else e = launch_staged<float, 3>(a, grid, st);
    }
    ++launched;
    return e == cudaSuccess ? launched : -1;
}

}  // namespace sqc
