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

// One slot held by a lane: its group, amplitude and presence, where it lives (b = -1 for a
// group absent at the start of the pass) and whether the pass changed it.
template <class T> struct Val {
    unsigned long long G;
    long long b;
    Cx<T> amp;
    bool pres, pres0, dirty;
};

struct GateHead {
    uint32_t kind, target, flip, credit;
    unsigned long long ctrl, cval;
};

__device__ __forceinline__ GateHead gate_head(const GateDesc* g) {
    GateHead h;
    h.kind = __ldg(&g->kind);
    h.target = __ldg(&g->target);
    h.flip = __ldg(&g->flip);
    h.credit = __ldg(&g->pad);
    h.ctrl = __ldg(&g->ctrl);
    h.cval = __ldg(&g->cval);
    return h;
}

// One streamable gate on one held slot. `off` is the lane distance to the partner slot
// (1 << q for q < 4, inside the half-warp) or 0 for a diagonal gate on a qubit >= 4.
template <class T>
__device__ __forceinline__ void gate_step(const GateDesc* g, const GateHead& h, int off, Val<T>& v, int j,
                                          const PruneBits& pb) {
    const unsigned long long key = (v.G << kSlotBits) | (unsigned long long)j;
    const bool sat = (key & h.ctrl) == h.cval;
    const bool bit = (((key >> h.target) & 1ULL) != 0) != (h.flip != 0);
    if (off) {
        Cx<T> pa;
        pa.r = __shfl_xor_sync(kFull, v.amp.r, off);
        pa.i = __shfl_xor_sync(kFull, v.amp.i, off);
        const bool pp = __shfl_xor_sync(kFull, (int)v.pres, off) != 0;
        if (is_swap(h.kind)) {
            if (sat) {
                v.amp = swap_update<T>(h.kind, bit, pa);
                v.pres = pp;
                v.dirty = true;
            }
        } else if (is_branch(h.kind)) {
            const bool any = v.pres || pp;
            if (__any_sync(kFull, sat && any)) {
                const Cx<T> o = branch_update<T>(h.kind, g, bit, v.amp, pa);
                if (sat) {
                    const bool keep = any && !negligible(o, pb);
                    v.pres = keep;
                    v.amp = keep ? o : czero<T>();
                    v.dirty = true;
                }
            }
        } else {
            const bool need = sat && v.pres && (bit || !is_one_sided(h.kind));
            if (__any_sync(kFull, need)) {
                const Cx<T> o = diag_update<T>(h.kind, g, bit, v.amp);
                if (need) { v.amp = o; v.dirty = true; }
            }
        }
        return;
    }
    const bool need = sat && v.pres && (bit || !is_one_sided(h.kind));
    if (__any_sync(kFull, need)) {
        const Cx<T> o = diag_update<T>(h.kind, g, bit, v.amp);
        if (need) { v.amp = o; v.dirty = true; }
    }
}

// The cross-group gate of a pair pass, lane-local: a = slot of G0 (stored bit 0), b = slot of G1.
template <class T>
__device__ __forceinline__ void pair_step(const GateDesc* g, const GateHead& h, Val<T>& a, Val<T>& b, int j,
                                          const PruneBits& pb) {
    const unsigned long long key = (a.G << kSlotBits) | (unsigned long long)j;
    const bool sat = (key & h.ctrl) == h.cval;
    const bool bit_a = h.flip != 0, bit_b = !bit_a;
    if (is_swap(h.kind)) {
        if (sat) {
            const Cx<T> na = swap_update<T>(h.kind, bit_a, b.amp), nb = swap_update<T>(h.kind, bit_b, a.amp);
            const bool pa = b.pres, pbr = a.pres;
            a.amp = na; b.amp = nb;
            a.pres = pa; b.pres = pbr;
            a.dirty = b.dirty = true;
        }
        return;
    }
    const bool any = a.pres || b.pres;
    if (__any_sync(kFull, sat && any)) {
        const Cx<T> oa = branch_update<T>(h.kind, g, bit_a, a.amp, b.amp);
        const Cx<T> ob = branch_update<T>(h.kind, g, bit_b, b.amp, a.amp);
        if (sat) {
            const bool ka = any && !negligible(oa, pb), kb = any && !negligible(ob, pb);
            a.pres = ka; a.amp = ka ? oa : czero<T>();
            b.pres = kb; b.amp = kb ? ob : czero<T>();
            a.dirty = b.dirty = true;
        }
    }
}

// Apply gates [g0, g1) to the two held slots; in a pair pass the first gate pairs them.
// Lane 0 accumulates the amp-update count: every gate is credited with the present slots
// it sees, and host-resolved gates recorded in a descriptor's credit with the same count.
template <class T>
__device__ __forceinline__ void run_gates(const GateDesc* __restrict__ gates, uint32_t g0, uint32_t g1,
                                          bool pair_first, Val<T>& a, Val<T>& b, int lane, const PruneBits& pb,
                                          unsigned long long& upd) {
    const int j = lane & 15;
    for (uint32_t gi = g0; gi < g1; ++gi) {
        const GateDesc* g = gates + gi;
        const GateHead h = gate_head(g);
        const unsigned n = __popc(__ballot_sync(kFull, a.pres)) + __popc(__ballot_sync(kFull, b.pres));
        if (lane == 0) upd += (unsigned long long)n * (1ULL + h.credit);
        if (gi == g0 && pair_first) {
            pair_step<T>(g, h, a, b, j, pb);
            continue;
        }
        const int off = h.target < (uint32_t)kSlotBits ? (1 << h.target) : 0;
        gate_step<T>(g, h, off, a, j, pb);
        gate_step<T>(g, h, off, b, j, pb);
    }
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
        if (b < 0 && hm && j == 0) cb = claim_group(t, ep, v.G, status, &created);
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
            t.keys[s] = v.pres ? ((v.G << kSlotBits) | (unsigned long long)j) : empty_key(j);
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
    v.G = G;
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

}  // namespace
}  // namespace sqc
