// Many-circuit batch: one persistent kernel runs the passes of every circuit of a batch.
//
// Every circuit has its own table slice, control block and gate descriptors, planned on the
// host exactly as for a single state; the per-slot code (sqc_pass_dev.cuh) is the same, so a
// circuit's result is bit-identical to running it alone. Scheduling is per circuit: pass p
// is cut into chunks of list entries, and a warp takes chunk i of pass p with one atomicAdd
// on the circuit's scheduling word (pass, chunks, issued). The warp that finishes the last
// chunk of a pass publishes the pass (key count, list length, counters) and opens the next
// one. Circuits never wait for each other, so short and long circuits share the GPU without
// lockstep.
//
// This file is compiled with global loads defaulting to L2 (-dlcm=cg): a persistent kernel
// reads, in pass p + 1, buckets that other SMs wrote in pass p, and L1 is not coherent.
// Gate descriptors and the circuit array never change during a launch and are read through
// the read-only path (plain non-coherent loads, without the pass kernels' L1 priority hint).
//
// A warp that finds no work sleeps briefly and retries; after idle_limit_ns without work it
// records ST_TIMEOUT in the batch control block and returns (the limit is a batch option,
// 2 s by default); every warp returns at its next check of that status. Parking: when the batch has a
// deadline, a circuit whose pass ends after the deadline parks instead of opening its next
// pass; a later launch resumes it (used by the serving loop to admit new circuits).
#define SQC_DESC_EVICT_LAST 0
#include "sqc_batch.h"
#include "sqc_pass_dev.cuh"

namespace sqc {
namespace {

constexpr int kBatchThreads = 256;
// FP32 circuits read each pass's gates from a per-warp shared-memory copy (7% faster on the
// 256-circuit batch); FP64 circuits read them in place (their registers are tighter: the copy
// cost 4%).
template <class T> struct BatchStage { static constexpr bool kOn = sizeof(T) == 4; };
constexpr unsigned kIdleSleepNs = 1000;                       // back-off of a warp that found no work

__device__ __forceinline__ unsigned long long sched_word(unsigned long long pass, unsigned long long chunks) {
    return (pass << (2 * kSchedFieldBits)) | (chunks << kSchedFieldBits);
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Chunking of a pass over n list entries: entries per chunk (a multiple of 4, at least
// min_chunk, large enough that the pass has at most target chunks) and the chunk count.
__device__ __forceinline__ void chunking(unsigned long long n, unsigned min_chunk, unsigned target, unsigned* chunk,
                                         unsigned* total) {
    unsigned long long c = (n + target - 1) / target;
    c = (c + 3) & ~3ULL;
    if (c < min_chunk) c = min_chunk;
    *chunk = (unsigned)c;
    const unsigned long long t = (n + c - 1) / c;
    *total = (unsigned)(t ? t : 1);
}

// Stream pass over list entries [eb, ee): each warp step holds four entries (two per half).
template <class T>
__device__ __forceinline__ void stream_chunk(const TableDev& t, const GateDesc* gates, const SmemGate* sg, uint32_t g0,
                                             uint32_t g1,
                                             unsigned ep, Ctl* ctl, unsigned long long eb, unsigned long long ee,
                                             const PruneBits& pb, unsigned long long& cnt_nnz,
                                             unsigned long long& cnt_empty, unsigned long long& upd) {
    const int lane = threadIdx.x & 31, half = lane >> 4, j = lane & 15;
    Val<T> va, vb;
    for (unsigned long long e0 = eb; e0 < ee; e0 += 4) {
        const unsigned long long ea = e0 + 2 * half, ebb = ea + 1;
        const long long ba = ea < ee ? (long long)t.list[ea] : -1;
        const long long bb = ebb < ee ? (long long)t.list[ebb] : -1;
        const unsigned long long Ga = ba >= 0 ? load_hdr(t.hdr + ba).group : 0ULL;
        const unsigned long long Gb = bb >= 0 ? load_hdr(t.hdr + bb).group : 0ULL;
        load_val_g<T>(t, va, Ga, ba, j);
        load_val_g<T>(t, vb, Gb, bb, j);
        if constexpr (BatchStage<T>::kOn) run_gates_s<T, false>(sg, gates, g0, g1, va, vb, lane, pb, upd);
        else run_gates<T, false>(gates, g0, g1, va, vb, lane, pb, upd);
        write_val<T>(t, ep, va, lane, &ctl->status, cnt_nnz, cnt_empty);
        write_val<T>(t, ep, vb, lane, &ctl->status, cnt_nnz, cnt_empty);
    }
}

// Pass that pairs groups over list entries [eb, ee), four entries at a time (units4 and
// run_units4 of sqc_pass_dev.cuh).
template <class T, int NX>
__device__ __forceinline__ void unit_chunk(const TableDev& t, const GateDesc* gates, const SmemGate* sg, uint32_t g0,
                                           uint32_t g1,
                                           uint32_t q1, uint32_t q2, unsigned ep, Ctl* ctl, unsigned long long eb,
                                           unsigned long long ee, const PruneBits& pb, unsigned long long& cnt_nnz,
                                           unsigned long long& cnt_empty, unsigned long long& upd) {
    const int lane = threadIdx.x & 31;
    const unsigned long long m1 = 1ULL << (q1 - kSlotBits);
    const unsigned long long m2 = NX == 2 ? 1ULL << (q2 - kSlotBits) : 0ULL;
    Val<T> va, vb;
    for (unsigned long long e0 = eb; e0 < ee; e0 += 4) {
        long long mb;
        unsigned long long G0;
        const unsigned om = units4<NX>(t, ep, e0, ee, m1, m2, lane, &mb, &G0);
        run_units4<T, NX, false, BatchStage<T>::kOn>(t, ep, ctl, gates, sg, g0, g1, m1, m2, om, mb, G0, lane, pb, va,
                                                     vb, cnt_nnz, cnt_empty, upd);
    }
}

// Lane 0, after the last chunk of pass p of circuit c: publish the pass and open the next
// one (or finish / park / fail the circuit).
__device__ void finish_circuit_pass(const BatchArgs& a, unsigned c, const BCirc& C, unsigned p) {
    Ctl* ctl = a.ctl + c;
    BSched* s = a.sched + c;
    __threadfence();
    const unsigned long long nnz_in = *(volatile unsigned long long*)&ctl->nnz;
    const unsigned long long tn = atomicExch(&ctl->acc_nnz, 0ULL);
    const unsigned long long te = atomicExch(&ctl->acc_empty, 0ULL);
    const unsigned long long tu = atomicExch(&ctl->acc_upd, 0ULL);
    const BPass bp = C.passes[p];
    bool ok = *(volatile unsigned int*)&ctl->status == 0;
    if (ok) {
        ctl->nnz = tn;
        ctl->empty_groups = te;
        ctl->list_n = *(volatile unsigned long long*)&ctl->list_tail;
        ctl->amp_updates += tu;
        const unsigned long long A = a.amp_bytes;
        const unsigned long long ab = bp.keys_fixed ? nnz_in * (8ULL + 2ULL * A) : (nnz_in + tn) * (8ULL + A);
        ctl->alg_bytes += ab;
        if (bp.nx) ctl->alg_bytes_pair += ab;
        ctl->seq += 1;
    }
    const unsigned next = p + 1;
    unsigned state = BS_RUN;
    unsigned chunk = 0, total = 0;
    if (!ok) {
        state = BS_FAILED;
    } else if (next >= C.npasses) {
        state = BS_DONE;
    } else {
        const unsigned long long n = ctl->list_n;
        const BPass nxp = C.passes[next];
        const unsigned long long grown = umin64(C.bound, n << nxp.nx);
        if (nxp.nx && grown > C.max_groups) {   // the slice could overflow: stop before touching it
            atomicCAS(&ctl->status, 0u, (unsigned)ST_GROW);
            state = BS_FAILED;
        } else {
            chunking(n, a.min_chunk, a.target_chunks, &chunk, &total);
            const unsigned long long dl = *(volatile unsigned long long*)&a.bctl->deadline_ns;
            if (next >= s->limit || (dl && globaltimer() > dl)) state = BS_PARKED;
        }
    }
    s->done = 0;
    s->chunk = chunk;
    s->next_total = total;
    s->state = state;
    __threadfence();
    atomicExch(a.words + c, sched_word(next, state == BS_RUN ? total : 0));
    if (state != BS_RUN) atomicSub(&a.bctl->left, 1u);
    atomicAdd(&a.bctl->progress, 1ULL);
}

// MINB: blocks per SM the register allocation is sized for (3: 80 registers with a few
// spills; 2: no spills).
template <class T, int MINB>
__global__ void __launch_bounds__(kBatchThreads, MINB) batch_run_kernel(BatchArgs a) {
    __shared__ SmemGate sgw[kBatchThreads / 32][BatchStage<T>::kOn ? kMaxRun : 1];
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned c = a.n ? warp % a.n : 0;
    unsigned long long idle_since = 0;
    while (true) {
        if (*(volatile unsigned int*)&a.bctl->status) return;
        if (*(volatile unsigned int*)&a.bctl->left == 0) return;
        // look for a chunk, starting at the circuit this warp worked on last: the lanes read
        // the scheduling words of 32 consecutive circuits at a time; the first one with a
        // chunk left is tried with an atomicAdd by its lane
        bool found = false;
        unsigned fc = 0, fp = 0, fi = 0, ftot = 0;
        for (unsigned base = 0; base < a.n && !found; base += 32) {
            const unsigned i = base + lane;
            const unsigned cc = i < a.n ? (c + i) % a.n : 0;
            bool avail = false;
            if (i < a.n) {
                const unsigned long long w = *(volatile unsigned long long*)(a.words + cc);
                avail = (w & kSchedFieldMask) < ((w >> kSchedFieldBits) & kSchedFieldMask);
            }
            unsigned mask = __ballot_sync(kFull, avail);
            while (mask && !found) {
                const int l = __ffs(mask) - 1;
                mask &= mask - 1;
                unsigned ok = 0, op = 0, oi = 0, ot = 0;
                if (lane == l) {
                    const unsigned long long old = atomicAdd(a.words + cc, 1ULL);
                    ot = (unsigned)((old >> kSchedFieldBits) & kSchedFieldMask);
                    oi = (unsigned)(old & kSchedFieldMask);
                    op = (unsigned)(old >> (2 * kSchedFieldBits));
                    ok = oi < ot;
                }
                if (__shfl_sync(kFull, ok, l)) {
                    found = true;
                    fc = __shfl_sync(kFull, cc, l);
                    fp = __shfl_sync(kFull, op, l);
                    fi = __shfl_sync(kFull, oi, l);
                    ftot = __shfl_sync(kFull, ot, l);
                }
            }
        }
        if (!found) {
            if (lane == 0) {
                const unsigned long long now = globaltimer();
                if (!idle_since) idle_since = now;
                else if (now - idle_since > a.idle_limit_ns) atomicCAS(&a.bctl->status, 0u, (unsigned)ST_TIMEOUT);
            }
            __syncwarp();
            __nanosleep(kIdleSleepNs);
            continue;
        }
        idle_since = 0;
        c = fc;
        __threadfence();   // acquire: the previous pass of this circuit is visible
        const BCirc C = a.circ[fc];
        Ctl* ctl = a.ctl + fc;
        const BPass bp = C.passes[fp];
        const unsigned long long n = *(volatile unsigned long long*)&ctl->list_n;
        const unsigned chunk = *(volatile unsigned int*)&a.sched[fc].chunk;
        const unsigned ep = *(volatile unsigned int*)&ctl->epoch;
        const unsigned long long eb = (unsigned long long)fi * chunk;
        const unsigned long long ee = umin64(eb + chunk, n);
        unsigned long long cnt_nnz = 0, cnt_empty = 0, upd = 0;
        const unsigned cst = __shfl_sync(kFull, *(volatile unsigned int*)&ctl->status, 0);
        if (eb < ee && cst == 0) {
            // FP32: the pass's gates into this warp's shared-memory copy (they are read once per
            // slot held, and loads default to L2 in this file); FP64 reads them in place
            SmemGate* sg = BatchStage<T>::kOn ? sgw[threadIdx.x >> 5] : nullptr;
            if constexpr (BatchStage<T>::kOn) stage_gates_warp(sg, C.gates, bp.g0, bp.g1, lane);
            if (bp.nx == 1)
                unit_chunk<T, 1>(C.t, C.gates, sg, bp.g0, bp.g1, bp.q1, kNoQubit, ep, ctl, eb, ee, a.prune, cnt_nnz,
                                 cnt_empty, upd);
            else if (bp.nx == 2)
                unit_chunk<T, 2>(C.t, C.gates, sg, bp.g0, bp.g1, bp.q1, bp.q2, ep, ctl, eb, ee, a.prune, cnt_nnz,
                                 cnt_empty, upd);
            else
                stream_chunk<T>(C.t, C.gates, sg, bp.g0, bp.g1, ep, ctl, eb, ee, a.prune, cnt_nnz, cnt_empty, upd);
        }
        cnt_nnz = warp_sum(cnt_nnz);
        cnt_empty = warp_sum(cnt_empty);
        upd = warp_sum(upd);
        if (lane == 0) {
            if (cnt_nnz) atomicAdd(&ctl->acc_nnz, cnt_nnz);
            if (cnt_empty) atomicAdd(&ctl->acc_empty, cnt_empty);
            if (upd) atomicAdd(&ctl->acc_upd, upd);
            __threadfence();   // release: this chunk's writes before its completion
            const unsigned d = atomicAdd(&a.sched[fc].done, 1u);
            if (d == ftot - 1) finish_circuit_pass(a, fc, C, fp);
        }
        __syncwarp();
    }
}

// Start a launch: one warp per circuit. BC_INIT resets the circuit to |0...0> under a new
// epoch (all its slice's buckets become free) and opens pass 0; BC_RESUME reopens a parked
// circuit's pending pass; BC_KEEP leaves the circuit as it is. The new epoch is taken from
// the batch control block, so a captured launch sequence replays with fresh epochs.
__global__ void batch_begin_kernel(BatchArgs a, unsigned long long deadline_ns) {
    __shared__ unsigned ep_new;
    __shared__ unsigned running;
    __shared__ unsigned any_init;
    if (threadIdx.x == 0) {
        ep_new = a.bctl->epoch + 1;
        if (ep_new == 0) ep_new = 1;   // epoch 0 marks cleared headers: never a live one
        running = 0;
        any_init = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (unsigned c = w; c < a.n; c += nw) {
        const unsigned cmd = a.cmd[c];
        BSched* s = a.sched + c;
        Ctl* ctl = a.ctl + c;
        const BCirc C = a.circ[c];
        if (cmd == BC_INIT) {
            __shared__ long long sb[32];
            if (lane == 0) {
                any_init = 1;
                ctl->epoch = ep_new;
                ctl->status = 0;
                ctl->done = 0;
                ctl->acc_nnz = ctl->acc_empty = ctl->acc_upd = 0;
                ctl->seq = 0;
                ctl->amp_updates = 0;
                ctl->alg_bytes = 0;
                ctl->alg_bytes_pair = 0;
                ctl->out_count = 0;
                bool created;
                sb[w] = claim_group(C.t, ep_new, 0ULL, &ctl->status, &created);
            }
            __syncwarp();
            const long long b = sb[w];
            if (b >= 0 && lane < kSlots) {
                const size_t sl = (size_t)b * kSlots + lane;
                C.t.keys[sl] = lane == 0 ? 0ULL : empty_key(lane);
                if (lane == 0) {
                    if (a.amp_bytes == 16) reinterpret_cast<double2*>(C.t.amps)[sl] = make_double2(1.0, 0.0);
                    else reinterpret_cast<float2*>(C.t.amps)[sl] = make_float2(1.0f, 0.0f);
                }
            }
            __syncwarp();
            if (lane == 0) {
                C.t.list[0] = (unsigned)(b >= 0 ? b : 0);
                ctl->list_n = ctl->list_tail = b >= 0 ? 1 : 0;
                ctl->nnz = b >= 0 ? 1 : 0;
                ctl->empty_groups = 0;
                const unsigned lim = a.limit[c];
                s->limit = lim;
                s->done = 0;
                unsigned chunk, total;
                chunking(ctl->list_n, a.min_chunk, a.target_chunks, &chunk, &total);
                s->chunk = chunk;
                s->next_total = total;
                const bool run = b >= 0 && C.npasses > 0 && lim > 0;
                s->state = run ? BS_RUN : (b >= 0 ? (C.npasses == 0 ? BS_DONE : BS_PARKED) : BS_FAILED);
                a.words[c] = sched_word(0, run ? total : 0);
                if (run) atomicAdd(&running, 1u);
            }
        } else if (cmd == BC_RESUME) {
            if (lane == 0) {
                const unsigned long long w0 = a.words[c];
                const unsigned p = (unsigned)(w0 >> (2 * kSchedFieldBits));
                s->limit = a.limit[c];
                if (s->state == BS_PARKED && p < s->limit && ctl->status == 0) {
                    s->state = BS_RUN;
                    s->done = 0;
                    a.words[c] = sched_word(p, s->next_total);
                    atomicAdd(&running, 1u);
                }
            }
        } else if (lane == 0 && s->state == BS_RUN) {
            atomicAdd(&running, 1u);   // kept running circuits still count
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (any_init) a.bctl->epoch = ep_new;
        a.bctl->status = 0;
        a.bctl->left = running;
        a.bctl->deadline_ns = deadline_ns ? globaltimer() + deadline_ns : 0ULL;
        a.bctl->progress = 0;
    }
}

}  // namespace

// Blocks per SM that fit for the variant a launch of `blocks_per_sm` (0: most) would use.
int batch_residency(bool dbl, int blocks_per_sm) {
    static int cache[2][2] = {{0, 0}, {0, 0}};
    const int v = blocks_per_sm == 0 || blocks_per_sm >= 3 ? 1 : 0;
    int& c = cache[dbl ? 1 : 0][v];
    if (!c) {
        int n = 0;
        if (dbl && v) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_run_kernel<double, 3>, kBatchThreads, 0);
        else if (dbl) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_run_kernel<double, 2>, kBatchThreads, 0);
        else if (v) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_run_kernel<float, 3>, kBatchThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_run_kernel<float, 2>, kBatchThreads, 0);
        c = n > 0 ? n : 1;
    }
    return c;
}

cudaError_t launch_batch(const BatchArgs& a, bool dbl, int grid, int blocks_per_sm, unsigned long long deadline_ns,
                         cudaStream_t st) {
    batch_begin_kernel<<<1, 1024, 0, st>>>(a, deadline_ns);
    const bool v3 = blocks_per_sm == 0 || blocks_per_sm >= 3;
    if (dbl) {
        if (v3) batch_run_kernel<double, 3><<<grid, kBatchThreads, 0, st>>>(a);
        else batch_run_kernel<double, 2><<<grid, kBatchThreads, 0, st>>>(a);
    } else {
        if (v3) batch_run_kernel<float, 3><<<grid, kBatchThreads, 0, st>>>(a);
        else batch_run_kernel<float, 2><<<grid, kBatchThreads, 0, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace sqc
