// Bookkeeping kernels of the sparse statevector engine (sm_103a): reset, loading a state,
// counting, readout, norm, state comparison and table rebuild. All walk the list of live
// buckets. The gate passes are in sqc_pass.cu.
#include "sqc_kernels.h"
#include "sqc_exact.cuh"

#include <algorithm>

namespace sqc {

namespace {

template <class T> struct AmpT;
template <> struct AmpT<double> { using V = double2; };
template <> struct AmpT<float> { using V = float2; };

template <class T>
__device__ __forceinline__ Cx<T> load_amp(const void* amps, size_t s) {
    const typename AmpT<T>::V v = reinterpret_cast<const typename AmpT<T>::V*>(amps)[s];
    return Cx<T>{v.x, v.y};
}
template <class T>
__device__ __forceinline__ void store_amp(void* amps, size_t s, Cx<T> a) {
    typename AmpT<T>::V v;
    v.x = a.r;
    v.y = a.i;
    reinterpret_cast<typename AmpT<T>::V*>(amps)[s] = v;
}
__device__ __forceinline__ Cx<double> load_amp_any(const void* amps, size_t s, bool dbl) {
    if (dbl) { const double2 v = reinterpret_cast<const double2*>(amps)[s]; return Cx<double>{v.x, v.y}; }
    const float2 v = reinterpret_cast<const float2*>(amps)[s];
    return Cx<double>{(double)v.x, (double)v.y};
}

template <class T> __device__ __forceinline__ Cx<T> czero() { return Cx<T>{T(0), T(0)}; }

__device__ __forceinline__ bool slot_present(unsigned long long key, int j) { return (int)(key & 15ULL) == j; }

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// |0...0>: new epoch (every bucket becomes free), claim group 0, store key 0 with amplitude 1.
__global__ void set_zero_kernel(TableDev t, Ctl* ctl, int dbl) {
    const int lane = threadIdx.x;
    __shared__ long long sb;
    if (lane == 0) {
        ctl->epoch += 1;
        ctl->status = 0;
        ctl->done = 0;
        ctl->work = 0;
        ctl->units_n = 0;
        ctl->acc_nnz = ctl->acc_empty = ctl->acc_upd = 0;
        ctl->seq = 0;
        ctl->amp_updates = 0;
        ctl->alg_bytes = 0;
        ctl->alg_bytes_pair = 0;
        bool created;
        sb = claim_group(t, ctl->epoch, 0ULL, &ctl->status, &created);
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
    if (lane == 0) {
        t.list[0] = (unsigned)(b >= 0 ? b : 0);
        ctl->list_n = ctl->list_tail = b >= 0 ? 1 : 0;
        ctl->nnz = b >= 0 ? 1 : 0;
        ctl->empty_groups = 0;
    }
}

// set_state step 0: new epoch, counters reset (one thread).
__global__ void set_state_begin_kernel(Ctl* ctl) {
    ctl->epoch += 1;
    ctl->status = 0;
    ctl->done = 0;
    ctl->work = 0;
    ctl->units_n = 0;
    ctl->acc_nnz = ctl->acc_empty = ctl->acc_upd = 0;
    ctl->seq = 0;
    ctl->amp_updates = 0;
    ctl->alg_bytes = 0;
    ctl->alg_bytes_pair = 0;
    ctl->out_count = 0;
    ctl->list_n = ctl->list_tail = 0;
    ctl->nnz = 0;
    ctl->empty_groups = 0;
}

// set_state step 1: claim the bucket of every entry's group; the claimer appends it to the list.
__global__ void set_state_claim_kernel(const unsigned long long* __restrict__ keys, unsigned long long n,
                                       TableDev t, Ctl* ctl) {
    const unsigned ep = ctl->epoch;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        bool created;
        const long long b = claim_group(t, ep, keys[i] >> kSlotBits, &ctl->status, &created);
        if (created) t.list[atomicAdd(&ctl->list_tail, 1ULL)] = (unsigned)b;
    }
}

// set_state step 2: mark every slot of every listed bucket empty.
__global__ void set_state_clear_kernel(TableDev t, Ctl* ctl) {
    const unsigned long long n = ctl->list_tail;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned b = t.list[s >> kSlotBits];
        t.keys[(size_t)b * kSlots + (s & 15)] = empty_key((int)(s & 15));
    }
}

// set_state step 3: store every entry in its slot; a second store to a slot is a duplicate key.
__global__ void set_state_fill_kernel(const unsigned long long* __restrict__ keys, const double* __restrict__ re,
                                      const double* __restrict__ im, unsigned long long n, TableDev t, Ctl* ctl,
                                      int dbl) {
    const unsigned ep = ctl->epoch;
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

// set_state step 4 (one thread): commit the list.
__global__ void set_state_end_kernel(Ctl* ctl, unsigned long long n) {
    ctl->list_n = ctl->list_tail;
    ctl->nnz = n;
}

// Present keys and empty live buckets over the list, into ctl->acc_nnz / acc_empty (adds).
__global__ void count_kernel(TableDev t, Ctl* ctl) {
    const unsigned long long n = ctl->list_n;
    unsigned long long c = 0, e = 0;
    for (unsigned long long s0 = (unsigned long long)blockIdx.x * blockDim.x; s0 < n * kSlots;
         s0 += (unsigned long long)gridDim.x * blockDim.x) {   // same trip count for the whole block
        const unsigned long long s = s0 + threadIdx.x;
        const int j = (int)(s & 15);
        bool p = false;
        if (s < n * kSlots) p = slot_present(t.keys[(size_t)t.list[s >> kSlotBits] * kSlots + j], j);
        c += p;
        const unsigned grp = __ballot_sync(kFull, p);
        if (s < n * kSlots && j == 0 && ((grp >> (threadIdx.x & 16)) & 0xFFFFu) == 0) e += 1;
    }
    c = warp_sum(c);
    e = warp_sum(e);
    if ((threadIdx.x & 31) == 0) {
        if (c) atomicAdd(&ctl->acc_nnz, c);
        if (e) atomicAdd(&ctl->acc_empty, e);
    }
}

// Compact the present entries whose stored key matches (key & smask) == sval into
// (keys ^ frame, re, im). Each warp owns a contiguous range of list entries: it counts,
// reserves its span with one atomic, then writes. Entries beyond cap are counted but not
// written.
template <class T>
__global__ void readout_kernel(TableDev t, Ctl* ctl, unsigned long long frame, unsigned long long* okeys,
                               double* ore, double* oim, unsigned long long cap, int drop_negl, PruneBits pb,
                               unsigned long long range, unsigned long long smask, unsigned long long sval) {
    const unsigned long long n = ctl->list_n;
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long r0 = warp * range; r0 < n; r0 += nwarps * range) {
        const unsigned long long r1 = r0 + range < n ? r0 + range : n;
        unsigned long long cnt = 0;
        for (unsigned long long ee = r0; ee < r1; ee += 2) {   // same trip count in both halves
            const unsigned long long e = ee + half;
            bool keep = false;
            if (e < r1) {
                const size_t s = (size_t)t.list[e] * kSlots + j;
                const unsigned long long k = t.keys[s];
                keep = slot_present(k, j) && (k & smask) == sval;
                if (keep && drop_negl) keep = !negligible(load_amp<T>(t.amps, s), pb);
            }
            cnt += __popc(__ballot_sync(kFull, keep));
        }
        unsigned long long base = 0;
        if (lane == 0 && cnt) base = atomicAdd(&ctl->out_count, cnt);
        base = shfl64(base, 0);
        if (!cnt) continue;
        unsigned long long pos = base;
        for (unsigned long long ee = r0; ee < r1; ee += 2) {
            const unsigned long long e = ee + half;
            bool keep = false;
            size_t s = 0;
            if (e < r1) {
                s = (size_t)t.list[e] * kSlots + j;
                const unsigned long long k = t.keys[s];
                keep = slot_present(k, j) && (k & smask) == sval;
                if (keep && drop_negl) keep = !negligible(load_amp<T>(t.amps, s), pb);
            }
            const unsigned bal = __ballot_sync(kFull, keep);
            if (keep) {
                const unsigned long long at = pos + __popc(bal & ((1u << lane) - 1u));
                if (at < cap) {
                    const Cx<T> v = load_amp<T>(t.amps, s);
                    okeys[at] = t.keys[s] ^ frame;
                    ore[at] = (double)v.r;
                    oim[at] = (double)v.i;
                }
            }
            pos += __popc(bal);
        }
    }
}

// Sum of |a|^2 over the state, exactly (sqc_exact.cuh), into sums->c[SUM_NORM].
template <class T>
__global__ void norm_kernel(TableDev t, Ctl* ctl, ExactSums* sums) {
    const unsigned long long n = ctl->list_n;
    unsigned long long acc[kSumChunks] = {};
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const size_t slot = (size_t)t.list[s >> kSlotBits] * kSlots + (s & 15);
        if (!slot_present(t.keys[slot], (int)(s & 15))) continue;
        const Cx<T> v = load_amp<T>(t.amps, slot);
        const double r = (double)v.r, i = (double)v.i;
        exact_add_prod(acc, r, r);
        exact_add_prod(acc, i, i);
    }
    exact_flush(acc, sums->c[SUM_NORM]);
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double v) {
    atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// Amplitude of the key stored as sb in state B, if present.
__device__ __forceinline__ bool find_other(const TableDev& tb, unsigned ep_b, unsigned long long sb, bool dbl_b,
                                           Cx<double>* out) {
    const long long bb = lookup_group(tb, ep_b, sb >> kSlotBits);
    if (bb < 0) return false;
    const int j = (int)(sb & 15ULL);
    const size_t s = (size_t)bb * kSlots + j;
    if (!slot_present(tb.keys[s], j)) return false;
    *out = load_amp_any(tb.amps, s, dbl_b);
    return true;
}

// Over the keys of a, exactly (sqc_exact.cuh): PART 0 sums conj(b)*a (real part into
// SUM_ORE, imaginary into SUM_OIM), PART 1 sums |a|^2 (SUM_NA) and |b|^2 (SUM_NB) and takes the
// max |a-b| (a max does not depend on the order). Two accumulators per launch keep the
// registers in check. d = frame_a ^ frame_b translates a stored key of a into b's frame.
template <int PART>
__global__ void compare_a_kernel(TableDev ta, const Ctl* ca, int dbl_a, TableDev tb, const Ctl* cb, int dbl_b,
                                 unsigned long long d, Ctl* out, ExactSums* sums) {
    const unsigned long long n = ca->list_n;
    const unsigned ep_b = cb->epoch;
    unsigned long long s0[kSumChunks] = {}, s1[kSumChunks] = {};
    double mx = 0;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const size_t slot = (size_t)ta.list[s >> kSlotBits] * kSlots + (s & 15);
        const unsigned long long key = ta.keys[slot];
        if (!slot_present(key, (int)(s & 15))) continue;
        const Cx<double> va = load_amp_any(ta.amps, slot, dbl_a);
        Cx<double> vb{0.0, 0.0};
        find_other(tb, ep_b, key ^ d, dbl_b, &vb);
        if (PART == 0) {
            exact_add_prod(s0, vb.r, va.r);
            exact_add_prod(s0, vb.i, va.i);
            exact_add_prod(s1, vb.r, va.i);
            exact_add_prod(s1, -vb.i, va.r);
        } else {
            exact_add_prod(s0, va.r, va.r);
            exact_add_prod(s0, va.i, va.i);
            exact_add_prod(s1, vb.r, vb.r);
            exact_add_prod(s1, vb.i, vb.i);
            const double dr = va.r - vb.r, di = va.i - vb.i;
            mx = fmax(mx, sqrt(dr * dr + di * di));
        }
    }
    exact_flush(s0, sums->c[PART == 0 ? SUM_ORE : SUM_NA]);
    exact_flush(s1, sums->c[PART == 0 ? SUM_OIM : SUM_NB]);
    if (PART == 1) {
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(kFull, mx, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&out->acc_max, mx);
    }
}

// Keys of b absent from a: SUM_NB_ONLY += |b|^2 (exactly), max |b|.
__global__ void compare_b_kernel(TableDev ta, const Ctl* ca, TableDev tb, const Ctl* cb, int dbl_b,
                                 unsigned long long d, Ctl* out, ExactSums* sums) {
    const unsigned long long n = cb->list_n;
    const unsigned ep_a = ca->epoch;
    unsigned long long s0[kSumChunks] = {};
    double mx = 0;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const size_t slot = (size_t)tb.list[s >> kSlotBits] * kSlots + (s & 15);
        const unsigned long long key = tb.keys[slot];
        if (!slot_present(key, (int)(s & 15))) continue;
        Cx<double> dummy;
        if (find_other(ta, ep_a, key ^ d, true, &dummy)) continue;
        const Cx<double> vb = load_amp_any(tb.amps, slot, dbl_b);
        exact_add_prod(s0, vb.r, vb.r);
        exact_add_prod(s0, vb.i, vb.i);
        mx = fmax(mx, sqrt(vb.r * vb.r + vb.i * vb.i));
    }
    exact_flush(s0, sums->c[SUM_NB_ONLY]);
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(kFull, mx, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&out->acc_max, mx);
}

// Copy the live, non-empty buckets of the old table into a new one (fresh headers, epoch
// ep_new), rebuilding the list. Each group appears once, so each new bucket has one writer.
__global__ void rehash_kernel(TableDev told, unsigned long long n_old, TableDev tnew, unsigned ep_new,
                              int amp_bytes, Ctl* ctl) {
    const int lane = threadIdx.x & 31, j = lane & 15, half = lane >> 4;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long e0 = warp * 2; e0 < n_old; e0 += nwarps * 2) {
        const unsigned long long e = e0 + half;
        const bool in = e < n_old;
        const unsigned b = in ? told.list[e] : 0u;
        const size_t s = (size_t)b * kSlots + j;
        const unsigned long long k = in ? told.keys[s] : 0ULL;
        const bool p = in && slot_present(k, j);
        const unsigned bal = __ballot_sync(kFull, p);
        const bool keep = in && ((half ? (bal >> 16) : (bal & 0xFFFFu)) != 0);
        long long nbk = -1;
        bool created = false;
        if (keep && j == 0) nbk = claim_group(tnew, ep_new, load_hdr(told.hdr + b).group, &ctl->status, &created);
        nbk = (long long)shfl64((unsigned long long)nbk, half << 4);
        const long long fresh = (keep && j == 0 && nbk >= 0) ? nbk : -1;
        if (keep && nbk >= 0) {
            const size_t d = (size_t)nbk * kSlots + j;
            tnew.keys[d] = k;
            if (p) {
                if (amp_bytes == 16) reinterpret_cast<double2*>(tnew.amps)[d] = reinterpret_cast<const double2*>(told.amps)[s];
                else reinterpret_cast<float2*>(tnew.amps)[d] = reinterpret_cast<const float2*>(told.amps)[s];
            }
        }
        const unsigned fm = __ballot_sync(kFull, fresh >= 0);
        if (fm) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&ctl->list_tail, (unsigned long long)__popc(fm));
            base = shfl64(base, 0);
            if (fresh >= 0) tnew.list[base + __popc(fm & ((1u << lane) - 1u))] = (unsigned)fresh;
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

cudaError_t launch_set_zero(const TableDev& t, Ctl* ctl, bool dbl, cudaStream_t st) {
    set_zero_kernel<<<1, 32, 0, st>>>(t, ctl, dbl ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_set_state(const unsigned long long* keys, const double* re, const double* im,
                             unsigned long long n, const TableDev& t, Ctl* ctl, bool dbl, int sms,
                             cudaStream_t st) {
    set_state_begin_kernel<<<1, 1, 0, st>>>(ctl);
    const int ge = grid_for(n, kThreads, sms);
    if (n) {
        set_state_claim_kernel<<<ge, kThreads, 0, st>>>(keys, n, t, ctl);
        set_state_clear_kernel<<<grid_for(n * kSlots, kThreads, sms), kThreads, 0, st>>>(t, ctl);
        set_state_fill_kernel<<<ge, kThreads, 0, st>>>(keys, re, im, n, t, ctl, dbl ? 1 : 0);
    }
    set_state_end_kernel<<<1, 1, 0, st>>>(ctl, n);
    return cudaGetLastError();
}

cudaError_t launch_count(const TableDev& t, Ctl* ctl, unsigned long long list_hint, int sms, cudaStream_t st) {
    count_kernel<<<grid_for(list_hint * kSlots + 1, kThreads, sms), kThreads, 0, st>>>(t, ctl);
    return cudaGetLastError();
}

cudaError_t launch_readout(const TableDev& t, Ctl* ctl, unsigned long long list_hint, unsigned long long frame,
                           bool dbl, unsigned long long* okeys, double* ore, double* oim, unsigned long long cap,
                           bool drop_negl, PruneBits pb, int sms, cudaStream_t st, unsigned long long smask,
                           unsigned long long sval) {
    const unsigned long long range = 64;
    const int grid = grid_for((list_hint + range - 1) / range + 1, kThreads / 32, sms);
    if (dbl)
        readout_kernel<double><<<grid, kThreads, 0, st>>>(t, ctl, frame, okeys, ore, oim, cap, drop_negl, pb, range,
                                                           smask, sval);
    else
        readout_kernel<float><<<grid, kThreads, 0, st>>>(t, ctl, frame, okeys, ore, oim, cap, drop_negl, pb, range,
                                                          smask, sval);
    return cudaGetLastError();
}

cudaError_t launch_norm(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl, ExactSums* sums, int sms,
                        cudaStream_t st) {
    const int grid = grid_for(list_hint * kSlots + 1, kThreads, sms);
    if (dbl) norm_kernel<double><<<grid, kThreads, 0, st>>>(t, ctl, sums);
    else norm_kernel<float><<<grid, kThreads, 0, st>>>(t, ctl, sums);
    return cudaGetLastError();
}

cudaError_t launch_compare(const TableDev& ta, const Ctl* ca, unsigned long long hint_a, bool dbl_a,
                           const TableDev& tb, const Ctl* cb, unsigned long long hint_b, bool dbl_b,
                           unsigned long long d, Ctl* out, ExactSums* sums, int sms, cudaStream_t st) {
    const int ga = grid_for(hint_a * kSlots + 1, kThreads, sms);
    compare_a_kernel<0><<<ga, kThreads, 0, st>>>(ta, ca, dbl_a, tb, cb, dbl_b, d, out, sums);
    compare_a_kernel<1><<<ga, kThreads, 0, st>>>(ta, ca, dbl_a, tb, cb, dbl_b, d, out, sums);
    compare_b_kernel<<<grid_for(hint_b * kSlots + 1, kThreads, sms), kThreads, 0, st>>>(ta, ca, tb, cb, dbl_b, d, out,
                                                                                        sums);
    return cudaGetLastError();
}

// Throughput probe of the FP64 pipe: every thread runs eight independent chains of dependent
// fused multiply-adds (x = x * a + b), so the pipe, not latency, bounds it. The result is kept
// alive by a store no input can trigger.
__global__ void fp64_rate_kernel(double* sink, double a, double b, int iters) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = __fma_rn(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == -1.0) sink[0] = s;
}

cudaError_t measure_fp64_rate(int sms, double* fma_per_s) {
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&sink, sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = 0.f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {   // the first launch warms up
        cudaEventRecord(e0);
        fp64_rate_kernel<<<blocks, threads>>>(sink, 0.9999999, 1e-7, iters);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    *fma_per_s = (e == cudaSuccess && best > 0.f) ? (double)blocks * threads * iters * 8 / (best * 1e-3) : 0.0;
    return e;
}

cudaError_t launch_rehash(const TableDev& told, unsigned long long n_old, const TableDev& tnew, unsigned ep_new,
                          int amp_bytes, Ctl* ctl, int sms, cudaStream_t st) {
    const int grid = grid_for(n_old / 2 + 1, kThreads / 32, sms);
    rehash_kernel<<<grid, kThreads, 0, st>>>(told, n_old, tnew, ep_new, amp_bytes, ctl);
    return cudaGetLastError();
}

}  // namespace sqc
