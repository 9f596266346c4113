// Gate-pass and bookkeeping kernels of the sparse statevector engine (sm_103a).
//
// One gate pass reads the input table and writes a fresh output table. Two pass shapes:
//  * stream pass: a run of gates that never pair keys across 16-key groups -- diagonal
//    gates on any qubit, any gate on qubits 0..3 (the partner is in the same bucket and is
//    reached with a warp shuffle), and X/Y on a qubit >= 4 whose controls are all >= 4 (the
//    whole group moves to G ^ (1 << (q-4)) or stays). Each half-warp streams one bucket.
//  * pair pass: a gate whose partner key lives in another group (branching gate on a qubit
//    >= 4, or X/Y on a qubit >= 4 with a control below 4), followed by a stream run. A warp
//    takes the group pair (G0, G1 = G0 | m): lanes 0-15 hold G0's slots, 16-31 G1's; the
//    partner of every lane is lane ^ 16. The group with target bit 0 owns the pair; the
//    bit-1 group owns it only when its partner group is absent -- the reference's pair rule
//    (emulator/device/device_table_FC.cuh:62-110) lifted from keys to 16-key groups, which
//    yields the same pairs and the same per-key results.
// Every pair with at least one present member is read once and written once. Pruning
// follows the reference (emulator/device/device_data.cuh:108-156): branching gates drop
// negligible outputs, swap and diagonal gates keep every key.
#include "sqc_kernels.h"

namespace sqc {

namespace {

template <class T> struct AmpT;
template <> struct AmpT<double> { using V = double2; };
template <> struct AmpT<float> { using V = float2; };

template <class T>
__device__ __forceinline__ Cx<T> load_amp(const void* amps, size_t s) {
    typename AmpT<T>::V v = reinterpret_cast<const typename AmpT<T>::V*>(amps)[s];
    return Cx<T>{v.x, v.y};
}
template <class T>
__device__ __forceinline__ void store_amp(void* amps, size_t s, Cx<T> a) {
    typename AmpT<T>::V v;
    v.x = a.r; v.y = a.i;
    reinterpret_cast<typename AmpT<T>::V*>(amps)[s] = v;
}
__device__ __forceinline__ Cx<double> load_amp_any(const void* amps, size_t s, bool dbl) {
    if (dbl) { double2 v = reinterpret_cast<const double2*>(amps)[s]; return Cx<double>{v.x, v.y}; }
    float2 v = reinterpret_cast<const float2*>(amps)[s];
    return Cx<double>{(double)v.x, (double)v.y};
}

template <class T> __device__ __forceinline__ Cx<T> czero() { return Cx<T>{T(0), T(0)}; }

// One gate applied by one lane to its own slot. `off` is the lane distance to the partner
// (1 << q for q < 4 inside a half-warp, 16 across the two halves of a pair pass), or 0 for a
// gate that needs no partner (diagonal gate, or X/Y on a qubit >= 4 moving the whole group).
template <class T>
__device__ __forceinline__ void gate_step(const GateDesc* g, uint32_t kind, uint32_t target,
                                          unsigned long long ctrl, int off, unsigned long long& G, int j,
                                          Cx<T>& amp, bool& pres, const PruneBits& pb) {
    const unsigned long long key = (G << kSlotBits) | (unsigned long long)j;
    const bool sat = (key & ctrl) == ctrl;
    const bool bit = (key >> target) & 1ULL;
    if (off) {
        Cx<T> pa;
        pa.r = __shfl_xor_sync(kFull, amp.r, off);
        pa.i = __shfl_xor_sync(kFull, amp.i, off);
        const bool pp = __shfl_xor_sync(kFull, (int)pres, off) != 0;
        if (is_swap(kind)) {
            if (sat) { amp = swap_update<T>(kind, bit, pa); pres = pp; }
        } else if (is_branch(kind)) {
            const bool any = pres || pp;
            if (__any_sync(kFull, sat && any)) {
                const Cx<T> o = branch_update<T>(kind, g, bit, amp, pa);
                if (sat) {
                    const bool keep = any && !negligible(o, pb);
                    pres = keep;
                    amp = keep ? o : czero<T>();
                }
            }
        } else if (__any_sync(kFull, sat && pres)) {
            const Cx<T> o = diag_update<T>(kind, g, bit, amp);
            if (sat) amp = o;
        }
        return;
    }
    if (is_swap(kind)) {           // target >= 4, controls >= 4: uniform over the group
        if (sat) {
            G ^= 1ULL << (target - kSlotBits);
            amp = swap_update<T>(kind, !bit, amp);
        }
    } else if (__any_sync(kFull, sat && pres)) {
        const Cx<T> o = diag_update<T>(kind, g, bit, amp);
        if (sat) amp = o;
    }
}

// Apply gates [g0, g1) to the lane's slot. In a pair pass the first gate pairs the halves.
template <class T>
__device__ __forceinline__ void run_gates(const GateDesc* __restrict__ gates, uint32_t g0, uint32_t g1,
                                          bool pair_first, unsigned long long& G, int lane, Cx<T>& amp,
                                          bool& pres, const PruneBits& pb, unsigned long long& upd) {
    const int j = lane & 15;
    const unsigned hmask = lane < 16 ? 0x0000FFFFu : 0xFFFF0000u;
    for (uint32_t gi = g0; gi < g1; ++gi) {
        const GateDesc* g = gates + gi;
        const uint32_t kind = __ldg(&g->kind), target = __ldg(&g->target);
        const unsigned long long ctrl = __ldg(&g->ctrl);
        const unsigned bal = __ballot_sync(kFull, pres);
        if (j == 0) upd += __popc(bal & hmask);
        int off;
        if (gi == g0 && pair_first) off = 16;
        else if (target < (uint32_t)kSlotBits) off = 1 << target;
        else off = 0;
        gate_step<T>(g, kind, target, ctrl, off, G, j, amp, pres, pb);
    }
}

// Write one half-warp's group into the output table: claim its bucket, write all 16 keys
// (present key or EMPTY marker) and the present amplitudes. Nothing is written for a group
// with no present key.
template <class T>
__device__ __forceinline__ void write_group(const TableDev& tout, unsigned ep_out, unsigned long long G,
                                            int lane, bool act, Cx<T> amp, bool pres, unsigned int* status,
                                            unsigned long long& cnt_nnz, unsigned long long& cnt_groups) {
    const int j = lane & 15, half = lane >> 4;
    const unsigned bal = __ballot_sync(kFull, pres && act);
    const unsigned hm = half ? (bal >> 16) : (bal & 0xFFFFu);
    long long ob = -1;
    if (j == 0 && hm) ob = claim_group(tout, ep_out, G, status);
    ob = (long long)shfl64((unsigned long long)ob, half << 4);
    if (hm && ob >= 0) {
        const size_t s = (size_t)ob * kSlots + j;
        tout.keys[s] = pres ? ((G << kSlotBits) | (unsigned long long)j) : empty_key(j);
        if (pres) store_amp<T>(tout.amps, s, amp);
        if (j == 0) cnt_groups += 1;
        cnt_nnz += pres ? 1 : 0;
    }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// Block-reduce the pass counters and let the last block publish the pass: new epoch of the
// output table, its key and group counts, the pass counter. Skipped when a pass failed.
__device__ void finish_pass(Ctl* ctl, int p, unsigned ep_out, unsigned long long n, unsigned long long g,
                            unsigned long long u, unsigned long long nnz_in, bool keys_fixed, unsigned amp_bytes) {
    __shared__ unsigned long long red[3][kThreads / 32];
    __shared__ bool last;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    n = warp_sum(n); g = warp_sum(g); u = warp_sum(u);
    if (lane == 0) { red[0][w] = n; red[1][w] = g; red[2][w] = u; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bn = 0, bg = 0, bu = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { bn += red[0][i]; bg += red[1][i]; bu += red[2][i]; }
        if (bn) atomicAdd(&ctl->acc_nnz, bn);
        if (bg) atomicAdd(&ctl->acc_groups, bg);
        if (bu) atomicAdd(&ctl->acc_upd, bu);
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->done, 1u);
        last = prev == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const unsigned long long tn = atomicExch(&ctl->acc_nnz, 0ULL);
        const unsigned long long tg = atomicExch(&ctl->acc_groups, 0ULL);
        const unsigned long long tu = atomicExch(&ctl->acc_upd, 0ULL);
        if (*(volatile unsigned int*)&ctl->status == 0) {
            ctl->nnz[p ^ 1] = tn;
            ctl->groups[p ^ 1] = tg;
            ctl->epoch[p ^ 1] = ep_out;
            ctl->amp_updates += tu;
            ctl->alg_bytes += keys_fixed ? nnz_in * (8ULL + 2ULL * amp_bytes) : (nnz_in + tn) * (8ULL + amp_bytes);
            ctl->seq += 1;
        }
        ctl->done = 0;
        __threadfence();
    }
}

template <class T, bool PAIR>
__global__ void __launch_bounds__(kThreads, 4) pass_kernel(PassArgs a) {
    Ctl* ctl = a.ctl;
    if (*(volatile unsigned int*)&ctl->status) return;
    const int p = (int)a.parity;
    const unsigned ep_in = ctl->epoch[p];
    const unsigned ep_out = ctl->epoch[p ^ 1] + 1;
    const unsigned long long nnz_in = ctl->nnz[p];
    const TableDev tin = p ? a.tab[1] : a.tab[0];
    const TableDev tout = p ? a.tab[0] : a.tab[1];
    const unsigned long long nb = tin.mask + 1;
    const int lane = threadIdx.x & 31, half = lane >> 4, j = lane & 15;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long cnt_nnz = 0, cnt_groups = 0, upd = 0;

    for (unsigned long long base = warp * 32; base < nb; base += nwarps * 32) {
        const Header h = load_hdr(tin.hdr + base + lane);
        unsigned vm = __ballot_sync(kFull, h.epoch == ep_in);
        if (!PAIR) {
            while (vm) {
                const int i0 = __ffs(vm) - 1;
                vm &= vm - 1;
                int i1 = -1;
                if (vm) { i1 = __ffs(vm) - 1; vm &= vm - 1; }
                const int mi = half ? i1 : i0;
                const bool act = mi >= 0;
                const int src = act ? mi : i0;
                unsigned long long G = shfl64(h.group, src);
                const size_t s = (size_t)(base + src) * kSlots + j;
                const unsigned long long key = act ? tin.keys[s] : 0ULL;
                bool pres = act && (int)(key & 15ULL) == j;
                Cx<T> amp = pres ? load_amp<T>(tin.amps, s) : czero<T>();
                run_gates<T>(a.gates, a.g0, a.g1, false, G, lane, amp, pres, a.prune, upd);
                write_group<T>(tout, ep_out, G, lane, act, amp, pres, &ctl->status, cnt_nnz, cnt_groups);
            }
        } else {
            const uint32_t q = __ldg(&a.gates[a.g0].target);
            const unsigned long long m = 1ULL << (q - kSlotBits);
            while (vm) {
                const int bi = __ffs(vm) - 1;
                vm &= vm - 1;
                const unsigned long long G = shfl64(h.group, bi);
                const bool mine1 = (G & m) != 0;
                long long bp = -1;
                if (lane == 0) bp = lookup_group(tin, ep_in, G ^ m);
                bp = (long long)shfl64((unsigned long long)bp, 0);
                if (mine1 && bp >= 0) continue;     // the bit-0 group owns this pair
                const long long b = (long long)(base + bi);
                const long long mb = half ? (mine1 ? b : bp) : (mine1 ? -1 : b);
                unsigned long long Gh = half ? (G | m) : (G & ~m);
                const size_t s = (size_t)(mb < 0 ? 0 : mb) * kSlots + j;
                const unsigned long long key = mb >= 0 ? tin.keys[s] : 0ULL;
                bool pres = mb >= 0 && (int)(key & 15ULL) == j;
                Cx<T> amp = pres ? load_amp<T>(tin.amps, s) : czero<T>();
                run_gates<T>(a.gates, a.g0, a.g1, true, Gh, lane, amp, pres, a.prune, upd);
                write_group<T>(tout, ep_out, Gh, lane, true, amp, pres, &ctl->status, cnt_nnz, cnt_groups);
            }
        }
    }
    finish_pass(ctl, p, ep_out, cnt_nnz, cnt_groups, upd, nnz_in, a.keys_fixed != 0, a.amp_bytes);
}

// |0...0>: discard the state (both epochs advance past anything a failed pass may have
// claimed), claim group 0 in table p and store key 0 with amplitude 1. One warp.
__global__ void set_zero_kernel(TableDev t, Ctl* ctl, int p, int dbl) {
    const int lane = threadIdx.x;
    __shared__ long long sb;
    __shared__ unsigned sep;
    if (lane == 0) {
        ctl->epoch[0] += 2;
        ctl->epoch[1] += 2;
        ctl->status = 0;
        ctl->done = 0;
        ctl->acc_nnz = ctl->acc_groups = ctl->acc_upd = 0;
        ctl->seq = 0;
        ctl->amp_updates = 0;
        ctl->alg_bytes = 0;
        const unsigned ep = ctl->epoch[p] + 1;
        sep = ep;
        sb = claim_group(t, ep, 0ULL, &ctl->status);
    }
    __syncwarp();
    const long long b = sb;
    if (b >= 0 && lane < kSlots) {
        const size_t s = (size_t)b * kSlots + lane;
        t.keys[s] = lane == 0 ? 0ULL : empty_key(lane);
        if (lane == 0) {
            if (dbl) reinterpret_cast<double2*>(t.amps)[s] = make_double2(1.0, 0.0);
            else reinterpret_cast<float2*>(t.amps)[s] = make_float2(1.0f, 0.0f);
        }
    }
    __syncwarp();
    if (lane == 0 && b >= 0) {
        ctl->epoch[p] = sep;
        ctl->nnz[p] = 1;
        ctl->groups[p] = 1;
        ctl->nnz[p ^ 1] = 0;
        ctl->groups[p ^ 1] = 0;
    }
}

// set_state step 0: reset the control block and advance the epochs (one thread).
__global__ void set_state_begin_kernel(Ctl* ctl, int p) {
    ctl->epoch[0] += 2;
    ctl->epoch[1] += 2;
    ctl->epoch[p] += 1;
    ctl->status = 0;
    ctl->done = 0;
    ctl->acc_nnz = ctl->acc_groups = ctl->acc_upd = 0;
    ctl->seq = 0;
    ctl->amp_updates = 0;
    ctl->alg_bytes = 0;
    ctl->out_count = 0;
}

// set_state step 1: claim the bucket of every entry's group (several entries may share one).
__global__ void set_state_claim_kernel(const unsigned long long* __restrict__ keys, unsigned long long n,
                                       TableDev t, Ctl* ctl, int p) {
    const unsigned ep = ctl->epoch[p];
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        claim_group(t, ep, keys[i] >> kSlotBits, &ctl->status);
}

// set_state step 2: mark every slot of every live bucket empty.
__global__ void set_state_clear_kernel(TableDev t, Ctl* ctl, int p) {
    const unsigned ep = ctl->epoch[p];
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < nslots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        if (load_hdr(t.hdr + (s >> kSlotBits)).epoch == ep) t.keys[s] = empty_key((int)(s & 15));
    }
}

// set_state step 3: store every entry in its slot; a second store to a slot is a duplicate key.
__global__ void set_state_fill_kernel(const unsigned long long* __restrict__ keys, const double* __restrict__ re,
                                      const double* __restrict__ im, unsigned long long n, TableDev t, Ctl* ctl,
                                      int p, int dbl) {
    const unsigned ep = ctl->epoch[p];
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        const long long b = lookup_group(t, ep, k >> kSlotBits);
        if (b < 0) { atomicCAS(&ctl->status, 0u, (unsigned)ST_TABLE_FULL); continue; }
        const int j = (int)(k & 15ULL);
        const size_t s = (size_t)b * kSlots + j;
        const unsigned long long old = atomicCAS(t.keys + s, empty_key(j), k);
        if (old != empty_key(j)) { atomicCAS(&ctl->status, 0u, (unsigned)ST_DUPLICATE); continue; }
        if (dbl) reinterpret_cast<double2*>(t.amps)[s] = make_double2(re[i], im[i]);
        else reinterpret_cast<float2*>(t.amps)[s] = make_float2((float)re[i], (float)im[i]);
    }
}

// Count live buckets and present keys of table p into ctl->nnz[p] / groups[p] (adds; the
// host zeroes them first).
__global__ void count_kernel(TableDev t, Ctl* ctl, int p) {
    const unsigned ep = ctl->epoch[p];
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    unsigned long long n = 0, g = 0;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < nslots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        if (load_hdr(t.hdr + (s >> kSlotBits)).epoch != ep) continue;
        const int j = (int)(s & 15);
        n += (int)(t.keys[s] & 15ULL) == j;
        g += j == 0;
    }
    n = warp_sum(n);
    g = warp_sum(g);
    if ((threadIdx.x & 31) == 0) {
        if (n) atomicAdd(&ctl->nnz[p], n);
        if (g) atomicAdd(&ctl->groups[p], g);
    }
}

// Compact the present entries of table p into (keys, re, im). Each warp owns a contiguous
// range of buckets: it counts, reserves its span with one atomic, then writes. Entries
// beyond cap are counted but not written.
template <class T>
__global__ void readout_kernel(TableDev t, Ctl* ctl, int p, unsigned long long* okeys, double* ore,
                               double* oim, unsigned long long cap, int drop_negl, PruneBits pb,
                               unsigned long long range) {
    const unsigned ep = ctl->epoch[p];
    const unsigned long long nb = t.mask + 1;
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long r0 = warp * range; r0 < nb; r0 += nwarps * range) {
        const unsigned long long r1 = r0 + range < nb ? r0 + range : nb;
        unsigned long long cnt = 0;
        for (unsigned long long bb = r0; bb < r1; bb += 2) {   // same trip count in both halves
            const unsigned long long b = bb + half;
            bool keep = false;
            if (b < r1 && load_hdr(t.hdr + b).epoch == ep) {
                const size_t s = (size_t)b * kSlots + j;
                keep = (int)(t.keys[s] & 15ULL) == j;
                if (keep && drop_negl) keep = !negligible(load_amp<T>(t.amps, s), pb);
            }
            cnt += __popc(__ballot_sync(kFull, keep));
        }
        // every lane holds the same total (each ballot is warp-wide); both halves counted
        cnt = __shfl_sync(kFull, cnt, 0);
        unsigned long long base = 0;
        if (lane == 0 && cnt) base = atomicAdd(&ctl->out_count, cnt);
        base = __shfl_sync(kFull, base, 0);
        if (!cnt) continue;
        unsigned long long pos = base;
        for (unsigned long long bb = r0; bb < r1; bb += 2) {
            const unsigned long long b = bb + half;
            bool keep = false;
            size_t s = 0;
            if (b < r1 && load_hdr(t.hdr + b).epoch == ep) {
                s = (size_t)b * kSlots + j;
                keep = (int)(t.keys[s] & 15ULL) == j;
                if (keep && drop_negl) keep = !negligible(load_amp<T>(t.amps, s), pb);
            }
            const unsigned bal = __ballot_sync(kFull, keep);
            if (keep) {
                const unsigned long long at = pos + __popc(bal & ((1u << lane) - 1u));
                if (at < cap) {
                    const Cx<T> v = load_amp<T>(t.amps, s);
                    okeys[at] = t.keys[s];
                    ore[at] = (double)v.r;
                    oim[at] = (double)v.i;
                }
            }
            pos += __popc(bal);
        }
    }
}

// Sum of |a|^2 over table p, accumulated in FP64, into ctl->acc[0].
template <class T>
__global__ void norm_kernel(TableDev t, Ctl* ctl, int p) {
    const unsigned ep = ctl->epoch[p];
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    double acc = 0.0;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < nslots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        if (load_hdr(t.hdr + (s >> kSlotBits)).epoch != ep) continue;
        if ((int)(t.keys[s] & 15ULL) != (int)(s & 15)) continue;
        const Cx<T> v = load_amp<T>(t.amps, s);
        const double r = (double)v.r, i = (double)v.i;
        acc = __fma_rn(r, r, __fma_rn(i, i, acc));
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(&ctl->acc[0], acc);
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double v) {
    atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// Overlap of state a with state b over the keys of a: acc[0..1] += conj(b)*a, acc[2] += |a|^2,
// acc[3] += |b|^2 (keys of a), max |a-b|. One warp per bucket of a (half-warps alternate).
__global__ void compare_a_kernel(TableDev ta, unsigned ep_a, int dbl_a, TableDev tb, unsigned ep_b, int dbl_b,
                                 Ctl* out) {
    const unsigned long long nb = ta.mask + 1;
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    double ore = 0, oim = 0, na = 0, nbb = 0, mx = 0;
    for (unsigned long long b0 = warp * 2; b0 < nb; b0 += nwarps * 2) {
        const unsigned long long b = b0 + half;
        const bool live = b < nb && load_hdr(ta.hdr + b).epoch == ep_a;
        long long bb = -1;
        if (live && j == 0) bb = lookup_group(tb, ep_b, load_hdr(ta.hdr + b).group);
        bb = (long long)shfl64((unsigned long long)bb, half << 4);
        if (!live) continue;
        const size_t s = (size_t)b * kSlots + j;
        if ((int)(ta.keys[s] & 15ULL) != j) continue;
        const Cx<double> va = load_amp_any(ta.amps, s, dbl_a);
        Cx<double> vb{0.0, 0.0};
        if (bb >= 0) {
            const size_t sb = (size_t)bb * kSlots + j;
            if ((int)(tb.keys[sb] & 15ULL) == j) vb = load_amp_any(tb.amps, sb, dbl_b);
        }
        ore += vb.r * va.r + vb.i * va.i;
        oim += vb.r * va.i - vb.i * va.r;
        na += va.r * va.r + va.i * va.i;
        nbb += vb.r * vb.r + vb.i * vb.i;
        const double dr = va.r - vb.r, di = va.i - vb.i;
        mx = fmax(mx, sqrt(dr * dr + di * di));
    }
    ore = warp_sum(ore); oim = warp_sum(oim); na = warp_sum(na); nbb = warp_sum(nbb);
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(kFull, mx, o));
    if (lane == 0) {
        atomicAdd(&out->acc[0], ore);
        atomicAdd(&out->acc[1], oim);
        atomicAdd(&out->acc[2], na);
        atomicAdd(&out->acc[3], nbb);
        atomic_max_nonneg(&out->acc_max, mx);
    }
}

// Keys of b absent from a: acc[4] += |b|^2, max |b|.
__global__ void compare_b_kernel(TableDev ta, unsigned ep_a, TableDev tb, unsigned ep_b, int dbl_b, Ctl* out) {
    const unsigned long long nb = tb.mask + 1;
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    double nbo = 0, mx = 0;
    for (unsigned long long b0 = warp * 2; b0 < nb; b0 += nwarps * 2) {
        const unsigned long long b = b0 + half;
        const bool live = b < nb && load_hdr(tb.hdr + b).epoch == ep_b;
        long long ba = -1;
        if (live && j == 0) ba = lookup_group(ta, ep_a, load_hdr(tb.hdr + b).group);
        ba = (long long)shfl64((unsigned long long)ba, half << 4);
        if (!live) continue;
        const size_t s = (size_t)b * kSlots + j;
        if ((int)(tb.keys[s] & 15ULL) != j) continue;
        bool in_a = false;
        if (ba >= 0) in_a = (int)(ta.keys[(size_t)ba * kSlots + j] & 15ULL) == j;
        if (in_a) continue;
        const Cx<double> vb = load_amp_any(tb.amps, s, dbl_b);
        nbo += vb.r * vb.r + vb.i * vb.i;
        mx = fmax(mx, sqrt(vb.r * vb.r + vb.i * vb.i));
    }
    nbo = warp_sum(nbo);
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(kFull, mx, o));
    if (lane == 0) {
        atomicAdd(&out->acc[4], nbo);
        atomic_max_nonneg(&out->acc_max, mx);
    }
}

// Move the content of an old table into a larger new one (fresh headers, epoch ep_new).
// Every group appears once in the old table, so each new bucket has one writer.
__global__ void rehash_kernel(TableDev told, unsigned ep_old, TableDev tnew, unsigned ep_new, int amp_bytes,
                              Ctl* ctl) {
    const unsigned long long nb = told.mask + 1;
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long b0 = warp * 2; b0 < nb; b0 += nwarps * 2) {
        const unsigned long long b = b0 + half;
        const Header h = b < nb ? load_hdr(told.hdr + b) : Header{0, 0, 0};
        const bool live = b < nb && h.epoch == ep_old;
        long long nbk = -1;
        if (live && j == 0) nbk = claim_group(tnew, ep_new, h.group, &ctl->status);
        nbk = (long long)shfl64((unsigned long long)nbk, half << 4);
        if (!live || nbk < 0) continue;
        const size_t s = (size_t)b * kSlots + j, d = (size_t)nbk * kSlots + j;
        const unsigned long long k = told.keys[s];
        tnew.keys[d] = k;
        if ((int)(k & 15ULL) == j) {
            if (amp_bytes == 16) reinterpret_cast<double2*>(tnew.amps)[d] = reinterpret_cast<const double2*>(told.amps)[s];
            else reinterpret_cast<float2*>(tnew.amps)[d] = reinterpret_cast<const float2*>(told.amps)[s];
        }
    }
}

int grid_for(unsigned long long work_items, int per_block, int sms) {
    unsigned long long g = (work_items + per_block - 1) / per_block;
    const unsigned long long cap = (unsigned long long)sms * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

cudaError_t launch_pass(const PassArgs& a, bool dbl, int sms, cudaStream_t st) {
    const unsigned long long nb = a.tab[a.parity].mask + 1;
    const int grid = grid_for(nb / 32 + 1, kThreads / 32, sms);
    if (dbl) {
        if (a.pair) pass_kernel<double, true><<<grid, kThreads, 0, st>>>(a);
        else pass_kernel<double, false><<<grid, kThreads, 0, st>>>(a);
    } else {
        if (a.pair) pass_kernel<float, true><<<grid, kThreads, 0, st>>>(a);
        else pass_kernel<float, false><<<grid, kThreads, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_set_zero(const TableDev& t, Ctl* ctl, int p, bool dbl, cudaStream_t st) {
    set_zero_kernel<<<1, 32, 0, st>>>(t, ctl, p, dbl ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_set_state(const unsigned long long* keys, const double* re, const double* im,
                             unsigned long long n, const TableDev& t, Ctl* ctl, int p, bool dbl, int sms,
                             cudaStream_t st) {
    set_state_begin_kernel<<<1, 1, 0, st>>>(ctl, p);
    const int ge = grid_for(n, kThreads, sms);
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    const int gs = grid_for(nslots, kThreads, sms);
    if (n) set_state_claim_kernel<<<ge, kThreads, 0, st>>>(keys, n, t, ctl, p);
    set_state_clear_kernel<<<gs, kThreads, 0, st>>>(t, ctl, p);
    if (n) set_state_fill_kernel<<<ge, kThreads, 0, st>>>(keys, re, im, n, t, ctl, p, dbl ? 1 : 0);
    count_kernel<<<gs, kThreads, 0, st>>>(t, ctl, p);
    return cudaGetLastError();
}

cudaError_t launch_count(const TableDev& t, Ctl* ctl, int p, int sms, cudaStream_t st) {
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    count_kernel<<<grid_for(nslots, kThreads, sms), kThreads, 0, st>>>(t, ctl, p);
    return cudaGetLastError();
}

cudaError_t launch_readout(const TableDev& t, Ctl* ctl, int p, bool dbl, unsigned long long* okeys, double* ore,
                           double* oim, unsigned long long cap, bool drop_negl, PruneBits pb, int sms,
                           cudaStream_t st) {
    const unsigned long long nb = t.mask + 1;
    const unsigned long long range = 256;
    const int grid = grid_for((nb + range - 1) / range, kThreads / 32, sms);
    if (dbl) readout_kernel<double><<<grid, kThreads, 0, st>>>(t, ctl, p, okeys, ore, oim, cap, drop_negl, pb, range);
    else readout_kernel<float><<<grid, kThreads, 0, st>>>(t, ctl, p, okeys, ore, oim, cap, drop_negl, pb, range);
    return cudaGetLastError();
}

cudaError_t launch_norm(const TableDev& t, Ctl* ctl, int p, bool dbl, int sms, cudaStream_t st) {
    const unsigned long long nslots = (t.mask + 1) * kSlots;
    const int grid = grid_for(nslots, kThreads, sms);
    if (dbl) norm_kernel<double><<<grid, kThreads, 0, st>>>(t, ctl, p);
    else norm_kernel<float><<<grid, kThreads, 0, st>>>(t, ctl, p);
    return cudaGetLastError();
}

cudaError_t launch_compare(const TableDev& ta, unsigned ep_a, bool dbl_a, const TableDev& tb, unsigned ep_b,
                           bool dbl_b, Ctl* out, int sms, cudaStream_t st) {
    const int ga = grid_for((ta.mask + 1) / 2 + 1, kThreads / 32, sms);
    const int gb = grid_for((tb.mask + 1) / 2 + 1, kThreads / 32, sms);
    compare_a_kernel<<<ga, kThreads, 0, st>>>(ta, ep_a, dbl_a, tb, ep_b, dbl_b, out);
    compare_b_kernel<<<gb, kThreads, 0, st>>>(ta, ep_a, tb, ep_b, dbl_b, out);
    return cudaGetLastError();
}

cudaError_t launch_rehash(const TableDev& told, unsigned ep_old, const TableDev& tnew, unsigned ep_new,
                          int amp_bytes, Ctl* ctl, int sms, cudaStream_t st) {
    const int grid = grid_for((told.mask + 1) / 2 + 1, kThreads / 32, sms);
    rehash_kernel<<<grid, kThreads, 0, st>>>(told, ep_old, tnew, ep_new, amp_bytes, ctl);
    return cudaGetLastError();
}

}  // namespace sqc
