// Host engine: table sizing and growth, gate resolution and pass planning, descriptor upload,
// deferred status checks with replay. See sqc_engine.h.
#include "sqc_engine.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "sqc_exact.cuh"
#include "sqc_kernels.h"

namespace sqc {

namespace {

constexpr unsigned long long kMinBuckets = 64;
constexpr size_t kFlushAt = 1024;          // queued gates that trigger a launch
constexpr unsigned long long kTinyMaxList = 256;   // live buckets up to which a flush is one launch
constexpr size_t kDescInitial = 1 << 14;   // descriptors held between verified syncs
constexpr unsigned long long kEpochRestart = 0xFFFFFF00ULL;   // epochs before the headers are cleared
constexpr double kMaxLoad = 0.9;           // live buckets a pair pass may leave behind

unsigned long long pow2_at_least(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return p;
}


}  // namespace

Engine::~Engine() {
    if (stream_) cudaStreamSynchronize(stream_);
    if (copy_stream_) cudaStreamSynchronize(copy_stream_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    if (ev_gathered_) cudaEventDestroy(ev_gathered_);
    if (ev_copied_) cudaEventDestroy(ev_copied_);
    if (h_async_n_) cudaFreeHost(h_async_n_);
    free_table(&tab_);
    if (ctl_) cudaFree(ctl_);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    if (sums_) cudaFree(sums_);
    if (sums_host_) cudaFreeHost(sums_host_);
    if (d_desc_) cudaFree(d_desc_);
    if (h_desc_) cudaFreeHost(h_desc_);
    if (d_tiny_) cudaFree(d_tiny_);
    if (h_tiny_) cudaFreeHost(h_tiny_);
    if (d_rk_) cudaFree(d_rk_);
    if (d_rr_) cudaFree(d_rr_);
    if (d_ri_) cudaFree(d_ri_);
    for (void* p : {(void*)sort_.keys_out, (void*)sort_.re_out, (void*)sort_.im_out, (void*)sort_.idx_in,
                    (void*)sort_.idx_out, (void*)sort_.cum, sort_.tmp})
        if (p) cudaFree(p);
    for (cudaEvent_t e : ev_all_) cudaEventDestroy(e);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

int Engine::fail(int code, const std::string& msg) {
    err = msg;
    return code;
}

int Engine::cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return SQC_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SQC_ERR_OOM : SQC_ERR_CUDA;
}

// A launcher reported a failed launch: its error, or a generic one when the runtime holds none.
int Engine::launch_failed(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda(e, what);
    return fail(SQC_ERR_CUDA, std::string(what) + ": launch failed");
}

size_t Engine::bucket_bytes() const {
    return sizeof(Header) + kSlots * sizeof(unsigned long long) + kSlots * (dbl_ ? 16 : 8) + sizeof(unsigned) +
           sizeof(Unit);
}

unsigned long long Engine::max_groups() const { return (unsigned long long)(kMaxLoad * (double)tab_.nb); }

int Engine::init(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt) {
    sqc_options o;
    sqc_default_options(&o);
    if (opt) o = *opt;
    if (nq < 1 || nq > 64) return fail(SQC_ERR_ARG, "nq must be in 1..64");
    if (o.precision != SQC_FP64 && o.precision != SQC_FP32) return fail(SQC_ERR_ARG, "precision must be 64 or 32");
    if (!(o.prune_threshold > 0.0)) return fail(SQC_ERR_ARG, "prune_threshold must be > 0");
    if (!(o.load_factor > 0.0 && o.load_factor <= kMaxLoad)) return fail(SQC_ERR_ARG, "load_factor must be in (0, 0.9]");
    double reserve = 0.05;
    if (params) {
        if (params->N_devices != 1) return fail(SQC_ERR_NO_DEVICE, "one GPU per state: N_devices must be 1");
        reserve = params->coef_gpu_memory_reserve;
        if (!(reserve >= 0.0 && reserve < 1.0)) return fail(SQC_ERR_ARG, "coef_gpu_memory_reserve must be in [0, 1)");
    }
    nq_ = nq;
    dbl_ = o.precision == SQC_FP64;
    thr_ = o.prune_threshold;
    lf_ = o.load_factor;
    max_run_ = o.max_fused_gates ? std::min<uint32_t>(o.max_fused_gates, kMaxRun) : kMaxRun;
    if (o.max_cross_qubits > 3) return fail(SQC_ERR_ARG, "max_cross_qubits must be 0, 1, 2 or 3");
    // default: three for FP32 (octet passes measured 14% faster on the 40-qubit workload), two
    // for FP64 (octet passes hold four slots per lane, which halves the FP64 kernels' occupancy:
    // the direct kernel ran 10% slower on the 40-qubit workload; on the 64-qubit workload the
    // staged kernel gained 1.4% from the fewer passes, with 36% fewer bytes moved per circuit)
    max_nx_ = o.max_cross_qubits ? o.max_cross_qubits : (o.precision == SQC_FP32 ? 3 : 2);
    time_passes_ = o.time_passes != 0;
    dev_upd_only_ = o.device_updates_only != 0;
    sched_ = o.schedule_gates != 0;
    device_ = (int)o.device;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device_) return fail(SQC_ERR_NO_DEVICE, "no CUDA device");
    int rc = cuda(cudaSetDevice(device_), "cudaSetDevice");
    if (rc) return rc;
    cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_);
    size_t free_b = 0, total_b = 0;
    if ((rc = cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"))) return rc;
    budget_ = (size_t)((1.0 - reserve) * (double)total_b);

    if (o.stream) {
        stream_ = (cudaStream_t)o.stream;
    } else {
        if ((rc = cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
        own_stream_ = true;
    }

    std::memcpy(&prune_.d, &thr_, sizeof(double));
    float tf = (float)thr_;
    if ((double)tf >= thr_) tf = std::nextafter(tf, 0.0f);
    std::memcpy(&prune_.f, &tf, sizeof(float));

    if ((rc = cuda(cudaMalloc(&ctl_, sizeof(Ctl)), "cudaMalloc(ctl)"))) return rc;
    if ((rc = cuda(cudaMemset(ctl_, 0, sizeof(Ctl)), "cudaMemset(ctl)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&ctl_host_, sizeof(Ctl)), "cudaMallocHost(ctl)"))) return rc;
    if ((rc = cuda(cudaMalloc(&sums_, sizeof(ExactSums)), "cudaMalloc(sums)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&sums_host_, sizeof(ExactSums)), "cudaMallocHost(sums)"))) return rc;
    std::memset(ctl_host_, 0, sizeof(Ctl));
    if ((rc = ensure_desc(kDescInitial))) return rc;

    const unsigned long long nb =
        pow2_at_least(std::max<unsigned long long>(o.initial_buckets ? o.initial_buckets : 1024, kMinBuckets));
    if ((rc = alloc_table(nb, &tab_))) return rc;
    return set_zero();
}

int Engine::alloc_table(unsigned long long nb, HostTable* out) {
    if ((double)nb * bucket_bytes() > (double)budget_)
        return fail(SQC_ERR_BUDGET, "table memory would exceed the HBM budget");
    HostTable t;
    t.nb = nb;
    int rc;
    if ((rc = cuda(cudaMalloc(&t.hdr, nb * sizeof(Header)), "cudaMalloc(hdr)")) ||
        (rc = cuda(cudaMalloc(&t.keys, nb * kSlots * sizeof(unsigned long long)), "cudaMalloc(keys)")) ||
        (rc = cuda(cudaMalloc(&t.amps, nb * kSlots * (dbl_ ? 16 : 8)), "cudaMalloc(amps)")) ||
        (rc = cuda(cudaMalloc(&t.list, nb * sizeof(unsigned)), "cudaMalloc(list)")) ||
        (rc = cuda(cudaMalloc(&t.units, nb * sizeof(Unit)), "cudaMalloc(units)")) ||
        (rc = cuda(cudaMemsetAsync(t.hdr, 0, nb * sizeof(Header), stream_), "cudaMemset(hdr)"))) {
        free_table(&t);
        return rc;
    }
    *out = t;
    return SQC_OK;
}

void Engine::free_table(HostTable* t) {
    if (t->hdr) cudaFree(t->hdr);
    if (t->keys) cudaFree(t->keys);
    if (t->amps) cudaFree(t->amps);
    if (t->list) cudaFree(t->list);
    if (t->units) cudaFree(t->units);
    *t = HostTable();
}

TableDev Engine::dev() const {
    TableDev d;
    d.hdr = tab_.hdr;
    d.keys = tab_.keys;
    d.amps = tab_.amps;
    d.list = tab_.list;
    d.units = tab_.units;
    d.mask = tab_.nb - 1;
    return d;
}

int Engine::ensure_desc(size_t n) {
    if (n <= desc_cap_) return SQC_OK;
    const size_t cap = std::max(n, desc_cap_ * 2);
    if (d_desc_) cudaFree(d_desc_);
    if (h_desc_) cudaFreeHost(h_desc_);
    if (d_tiny_) cudaFree(d_tiny_);
    if (h_tiny_) cudaFreeHost(h_tiny_);
    d_desc_ = nullptr;
    h_desc_ = nullptr;
    d_tiny_ = nullptr;
    h_tiny_ = nullptr;
    desc_cap_ = 0;
    int rc;
    if ((rc = cuda(cudaMalloc(&d_desc_, cap * sizeof(GateDesc)), "cudaMalloc(desc)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&h_desc_, cap * sizeof(GateDesc)), "cudaMallocHost(desc)"))) return rc;
    // tiny-launch pass records, indexed like the descriptors (a flush has no more passes than gates)
    if ((rc = cuda(cudaMalloc(&d_tiny_, cap * sizeof(TinyPass)), "cudaMalloc(tiny)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&h_tiny_, cap * sizeof(TinyPass)), "cudaMallocHost(tiny)"))) return rc;
    desc_cap_ = cap;
    return SQC_OK;
}

int Engine::ensure_readout(size_t n) {
    if (n <= rcap_) return SQC_OK;
    if (async_pending_ && ev_copied_) {   // the buffers are about to be freed: the copy must be done
        int rc;
        if ((rc = cuda(cudaEventSynchronize(ev_copied_), "wait for the readout copy"))) return rc;
    }
    const size_t cap = std::max<size_t>(n, 1024);
    if (d_rk_) cudaFree(d_rk_);
    if (d_rr_) cudaFree(d_rr_);
    if (d_ri_) cudaFree(d_ri_);
    d_rk_ = nullptr; d_rr_ = nullptr; d_ri_ = nullptr; rcap_ = 0;
    int rc;
    if ((rc = cuda(cudaMalloc(&d_rk_, cap * 8), "cudaMalloc(readout)")) ||
        (rc = cuda(cudaMalloc(&d_rr_, cap * 8), "cudaMalloc(readout)")) ||
        (rc = cuda(cudaMalloc(&d_ri_, cap * 8), "cudaMalloc(readout)")))
        return rc;
    rcap_ = cap;
    return SQC_OK;
}

bool Engine::plan_gate(const sqc_gate& g, GateDesc* out) { return sqc::plan_gate(plan_, g, out); }

int Engine::set_zero() {
    pending_.clear();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    plan_ = Planner();
    snap_plan_ = plan_;
    snap_log_ = 0;
    host_upd_ = 0;
    list_hint_ = 1;
    int rc;
    if ((rc = next_epoch())) return rc;
    rc = cuda(launch_set_zero(dev(), ctl_, dbl_, stream_), "set_zero");
    ++launches_;
    return rc;
}

// set_zero and set_state move the table to a new epoch (their kernels bump Ctl::epoch), and
// headers of an older epoch read as empty. Before the 32-bit epoch could come back round to a
// value still stored in a header, the headers are cleared and the epoch starts over.
int Engine::next_epoch() {
    if (++epochs_ < kEpochRestart) return SQC_OK;
    epochs_ = 1;
    int rc;
    if ((rc = cuda(cudaMemsetAsync(tab_.hdr, 0, tab_.nb * sizeof(Header), stream_), "memset(headers)")) ||
        (rc = cuda(cudaMemsetAsync(&ctl_->epoch, 0, sizeof(ctl_->epoch), stream_), "memset(epoch)")))
        return rc;
    return SQC_OK;
}

int Engine::set_state(const uint64_t* keys, const double* re, const double* im, uint64_t n,
                      const KeySummary* known) {
    if (n && (!keys || !re || !im)) return fail(SQC_ERR_ARG, "null array");
    unsigned long long all_and = ~0ULL, all_or = 0, groups = 0;
    if (known) {
        all_and = known->all_and;
        all_or = known->all_or;
        groups = known->groups;
        if (nq_ < 64 && (all_or >> nq_)) return fail(SQC_ERR_ARG, "key does not fit in nq bits");
    } else {
        for (uint64_t i = 0; i < n; ++i) {
            if (nq_ < 64 && (keys[i] >> nq_)) return fail(SQC_ERR_ARG, "key does not fit in nq bits");
            all_and &= keys[i];
            all_or |= keys[i];
        }
        // groups in the input, counted as changes of key >> 4 along the array: exact when each
        // group's keys are contiguous (as readouts emit them), an upper bound otherwise
        unsigned long long prev = ~0ULL;
        for (uint64_t i = 0; i < n; ++i) {
            const unsigned long long g = keys[i] >> kSlotBits;
            groups += g != prev ? 1 : 0;
            prev = g;
        }
    }
    int rc;
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    pending_.clear();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    const unsigned long long need =
        pow2_at_least(std::max<unsigned long long>(kMinBuckets, (unsigned long long)std::ceil((double)groups / lf_)));
    if (need > tab_.nb) {
        HostTable nt;
        if ((rc = alloc_table(need, &nt))) return rc;
        free_table(&tab_);
        tab_ = nt;
    }
    if ((rc = ensure_readout(n))) return rc;
    if ((rc = readout_buffers_free())) return rc;
    if (n) {
        if ((rc = cuda(cudaMemcpyAsync(d_rk_, keys, n * 8, cudaMemcpyHostToDevice, stream_), "H2D keys")) ||
            (rc = cuda(cudaMemcpyAsync(d_rr_, re, n * 8, cudaMemcpyHostToDevice, stream_), "H2D re")) ||
            (rc = cuda(cudaMemcpyAsync(d_ri_, im, n * 8, cudaMemcpyHostToDevice, stream_), "H2D im")))
            return rc;
    }
    plan_ = Planner();
    if (n) {
        plan_.kmask = ~(all_and ^ all_or);
        plan_.kval = all_and & plan_.kmask;
    }
    snap_plan_ = plan_;
    snap_log_ = 0;
    host_upd_ = 0;
    list_hint_ = std::max<unsigned long long>(n, 1);
    if ((rc = next_epoch())) return rc;
    rc = cuda(launch_set_state(d_rk_, d_rr_, d_ri_, n, dev(), ctl_, dbl_, sms_, stream_), "set_state");
    launches_ += n ? 5 : 2;
    if (rc) return rc;
    if ((rc = read_ctl())) return rc;
    if (ctl_host_->status != ST_OK) {
        const bool dup = ctl_host_->status == ST_DUPLICATE;
        set_zero();
        return dup ? fail(SQC_ERR_ARG, "duplicate key in set_state") : fail(SQC_ERR_TABLE_FULL, "set_state: table full");
    }
    seq_verified_ = ctl_host_->seq;
    list_hint_ = std::max<unsigned long long>(ctl_host_->list_n, 1);
    return SQC_OK;
}

int Engine::apply(const sqc_gate* gates, uint64_t n) {
    if (n && !gates) return fail(SQC_ERR_ARG, "null gate array");
    for (uint64_t i = 0; i < n; ++i) {
        if (const char* why = check_gate(gates[i], nq_)) return fail(SQC_ERR_ARG, why);
    }
    if (sched_ && n > 1 && n <= kScheduleMaxGates) {   // the call's gates in the order passes fuse better
        perm_.resize(n);
        schedule_gates(gates, n, max_nx_, max_run_, kScheduleWindow, perm_.data());
        for (uint64_t i = 0; i < n; ++i) pending_.push_back(gates[perm_[i]]);
    } else {
        pending_.insert(pending_.end(), gates, gates + n);
    }
    if (pending_.size() >= kFlushAt) return flush();
    return SQC_OK;
}

// Resolve the queued gates, split the device gates into passes and launch them. A pass is
// either a run of streamable gates, or one cross-group gate followed by such a run.
int Engine::flush(bool hold_last) {
    if (pending_.empty()) return SQC_OK;
    const size_t n = pending_.size();
    int rc;
    if (desc_used_ + n > desc_cap_) {
        std::vector<sqc_gate> keep;
        keep.swap(pending_);
        if ((rc = sync())) {   // verifies everything launched, resets desc_used_
            pending_.insert(pending_.end(), keep.begin(), keep.end());   // keep them queued
            return rc;
        }
        pending_.swap(keep);
        if ((rc = ensure_desc(n))) return rc;
    }
    const size_t log_base = log_.size();
    log_.insert(log_.end(), pending_.begin(), pending_.end());
    GateDesc* hd = h_desc_ + desc_used_;
    std::vector<size_t> src;
    std::vector<Planner> after;
    src.reserve(n);
    after.reserve(n);
    size_t nd = 0;
    for (size_t i = 0; i < n; ++i) {
        GateDesc d;
        if (!plan_gate(pending_[i], &d)) continue;
        d.pad = dev_upd_only_ ? 0u : plan_.credit;   // credit: host-resolved gates before it
        plan_.credit = 0;
        hd[nd++] = d;
        src.push_back(log_base + i);
        after.push_back(plan_);
    }
    gates_applied_ += n;
    pending_.clear();
    if (nd == 0) return SQC_OK;
    PassArgs a;
    std::memset(&a, 0, sizeof a);
    a.t = dev();
    a.ctl = ctl_;
    a.gates = d_desc_ + desc_used_;
    a.amp_bytes = dbl_ ? 16u : 8u;
    a.max_groups = max_groups();
    a.prune = prune_;
    struct Span {
        size_t g0, g1;
        uint32_t nx, q1, q2, q3;
        bool fixed;
    };
    std::vector<Span> spans;
    split_passes(hd, nd, max_run_, max_nx_,
                 [&](size_t g0, size_t g1, uint32_t nx, uint32_t q1, uint32_t q2, uint32_t q3, bool fixed) {
                     spans.push_back(Span{g0, g1, nx, q1, q2, q3, fixed});
                     encode_pass(hd, g0, g1, q1, q3);
                 });
    if (hold_last && spans.size() >= 2) {
        // the last pass's gates, and the host-resolved gates around them, go back to the queue;
        // the planner returns to its state after the last device gate that is launched
        const size_t last_src = src[spans.back().g0 - 1];   // log index of that gate
        const size_t keep = last_src + 1 - log_base;        // queued gates that stay launched
        pending_.assign(log_.begin() + (std::ptrdiff_t)(log_base + keep), log_.end());
        log_.resize(log_base + keep);
        gates_applied_ -= n - keep;
        plan_ = after[spans.back().g0 - 1];
        spans.pop_back();
    }
    if ((rc = cuda(cudaMemcpyAsync(d_desc_ + desc_used_, hd, nd * sizeof(GateDesc), cudaMemcpyHostToDevice, stream_),
                   "H2D gate descriptors")))
        return rc;
    cudaEvent_t ev_prev = nullptr;
    if (time_passes_ && (rc = record_event(&ev_prev))) return rc;
    // a tiny state runs the flush's passes in one single-block launch (tiny_kernel): the live
    // buckets every pass may reach stay few enough that launches would cost more than the work
    {
        unsigned long long h = list_hint_, hmax = list_hint_;
        for (const Span& sp : spans) {
            if (sp.nx) h = std::min<unsigned long long>(tab_.nb, std::min(h << sp.nx, group_bound(after[sp.g1 - 1], nq_)));
            hmax = std::max(hmax, h);
        }
        if (spans.size() >= 2 && tiny_table(tab_.nb) && hmax <= kTinyMaxList) {
            TinyPass* ht = h_tiny_ + desc_used_;
            bool any_pair = false;
            for (size_t k = 0; k < spans.size(); ++k) {
                const Span& sp = spans[k];
                TinyPass& q = ht[k];
                q.g0 = (uint32_t)sp.g0;
                q.g1 = (uint32_t)sp.g1;
                q.nx = sp.nx;
                q.q1 = sp.q1;
                q.q2 = sp.q2;
                q.q3 = sp.q3;
                q.keys_fixed = sp.fixed ? 1u : 0u;
                q.pad = 0;
                q.grow_bound = group_bound(after[sp.g1 - 1], nq_);
                any_pair = any_pair || sp.nx > 0;
            }
            if ((rc = cuda(cudaMemcpyAsync(d_tiny_ + desc_used_, ht, spans.size() * sizeof(TinyPass),
                                           cudaMemcpyHostToDevice, stream_), "H2D tiny passes")))
                return rc;
            if (launch_tiny(a, d_tiny_ + desc_used_, (uint32_t)spans.size(), dbl_, stream_) < 0)
                return launch_failed("tiny passes");
            if (time_passes_) {
                cudaEvent_t ev = nullptr;
                if ((rc = record_event(&ev))) return rc;
                timed_.push_back(TimedPass{ev_prev, ev, any_pair});
            }
            for (const Span& sp : spans) {
                passes_pair_ += sp.nx > 0 ? 1 : 0;
                passes_.push_back(PassRec{snap_log_, snap_plan_});
                snap_log_ = src[sp.g1 - 1] + 1;
                snap_plan_ = after[sp.g1 - 1];
                ++passes_run_;
            }
            ++launches_;
            list_hint_ = h;
            desc_used_ += nd;
            return SQC_OK;
        }
    }
    for (const Span& sp : spans) {
        const size_t i = sp.g1;
        a.g0 = (uint32_t)sp.g0;
        a.g1 = (uint32_t)sp.g1;
        a.nx = sp.nx;
        a.q1 = sp.q1;
        a.q2 = sp.q2;
        a.q3 = sp.q3;
        a.keys_fixed = sp.fixed ? 1u : 0u;
        a.grow_bound = group_bound(after[i - 1], nq_);
        if (sp.nx)
            list_hint_ = std::min<unsigned long long>(tab_.nb, std::min(list_hint_ << sp.nx, a.grow_bound));
        const int nl = launch_pass(a, list_hint_, dbl_, sms_, stream_);
        if (nl < 0) return launch_failed("gate pass");
        const bool pair = sp.nx > 0;
        if (time_passes_) {
            cudaEvent_t ev = nullptr;
            if ((rc = record_event(&ev))) return rc;
            timed_.push_back(TimedPass{ev_prev, ev, pair});
            ev_prev = ev;
        }
        passes_pair_ += pair ? 1 : 0;
        passes_.push_back(PassRec{snap_log_, snap_plan_});
        snap_log_ = src[i - 1] + 1;
        snap_plan_ = after[i - 1];
        launches_ += (uint64_t)nl;
        ++passes_run_;
    }
    desc_used_ += nd;
    return SQC_OK;
}

int Engine::read_sums() {
    int rc;
    if ((rc = cuda(cudaMemcpyAsync(sums_host_, sums_, sizeof(ExactSums), cudaMemcpyDeviceToHost, stream_), "D2H sums")))
        return rc;
    return cuda(cudaStreamSynchronize(stream_), "sync");
}

// The exact total of a fixed-point accumulator (sqc_exact.cuh), rounded to the nearest double.
double exact_sum_value(const unsigned long long* acc) {
    uint32_t limb[kSumChunks];
    unsigned __int128 carry = 0;
    for (int i = 0; i < kSumChunks; ++i) {   // carry the pieces into 32-bit limbs (mod 2^(32 kSumChunks))
        const unsigned __int128 v = (unsigned __int128)acc[i] + carry;
        limb[i] = (uint32_t)v;
        carry = v >> 32;
    }
    const bool neg = (limb[kSumChunks - 1] >> 31) != 0;   // two's complement sign
    if (neg) {
        uint64_t c = 1;
        for (int i = 0; i < kSumChunks; ++i) {
            const uint64_t v = (uint64_t)(uint32_t)~limb[i] + c;
            limb[i] = (uint32_t)v;
            c = v >> 32;
        }
    }
    int h = kSumChunks - 1;
    while (h >= 0 && !limb[h]) --h;
    if (h < 0) return 0.0;
    // the top three limbs, the rest as a sticky bit; round to 53 bits, ties to even
    unsigned __int128 w = ((unsigned __int128)limb[h] << 64) | ((unsigned __int128)(h >= 1 ? limb[h - 1] : 0u) << 32) |
                          (unsigned __int128)(h >= 2 ? limb[h - 2] : 0u);
    bool sticky = false;
    for (int i = 0; i < h - 2; ++i) sticky = sticky || limb[i] != 0;
    int scale = 32 * (h - 2) + kSumLsb;   // weight of w's least significant bit
    int bits = 0;
    for (unsigned __int128 t = w; t; t >>= 1) ++bits;
    uint64_t m = (uint64_t)w;
    if (bits > 53) {
        const int drop = bits - 53;
        const unsigned __int128 rem = w & (((unsigned __int128)1 << drop) - 1);
        const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
        m = (uint64_t)(w >> drop);
        if (rem > half || (rem == half && (sticky || (m & 1)))) ++m;
        scale += drop;
    }
    const double v = std::ldexp((double)m, scale);
    return neg ? -v : v;
}

int Engine::read_ctl() {
    int rc;
    if ((rc = cuda(cudaMemcpyAsync(ctl_host_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "D2H ctl")))
        return rc;
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    harvest_events();
    return SQC_OK;
}

// Record an event on the stream (from the free list, or a new one).
int Engine::record_event(cudaEvent_t* out) {
    cudaEvent_t e;
    if (!ev_free_.empty()) {
        e = ev_free_.back();
        ev_free_.pop_back();
    } else {
        int rc;
        if ((rc = cuda(cudaEventCreate(&e), "event create"))) return rc;
        ev_all_.push_back(e);
    }
    *out = e;
    return cuda(cudaEventRecord(e, stream_), "event record");
}

// After a stream synchronize: add the timed passes to the totals and recycle their events.
// An event that starts one pass and ends the previous one is recycled once.
void Engine::harvest_events() {
    if (timed_.empty()) return;
    for (const TimedPass& p : timed_) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.before, p.after) == cudaSuccess) {
            const uint64_t ns = (uint64_t)((double)ms * 1e6);
            if (p.pair) pass_ns_pair_ += ns;
            else pass_ns_stream_ += ns;
        }
    }
    std::vector<cudaEvent_t> used;
    used.reserve(2 * timed_.size());
    for (const TimedPass& p : timed_) {
        used.push_back(p.before);
        used.push_back(p.after);
    }
    std::sort(used.begin(), used.end());
    used.erase(std::unique(used.begin(), used.end()), used.end());
    ev_free_.insert(ev_free_.end(), used.begin(), used.end());
    timed_.clear();
    cudaGetLastError();
}

int Engine::sync() {
    int rc;
    for (int attempt = 0; attempt < 64; ++attempt) {
        if ((rc = flush())) return rc;
        if ((rc = read_ctl())) return rc;
        const unsigned st = ctl_host_->status;
        if (st == ST_OK) {
            if (!dev_upd_only_) host_upd_ += (unsigned long long)plan_.credit * ctl_host_->nnz;
            plan_.credit = 0;
            seq_verified_ = ctl_host_->seq;
            log_.clear();
            passes_.clear();
            desc_used_ = 0;
            snap_log_ = 0;
            snap_plan_ = plan_;
            list_hint_ = std::max<unsigned long long>(ctl_host_->list_n, 1);
            // many groups left without keys (pruned away): rebuild without them
            if (ctl_host_->list_n > 4096 && ctl_host_->empty_groups * 2 > ctl_host_->list_n) {
                if ((rc = rebuild(tab_.nb))) return rc;
            }
            return SQC_OK;
        }
        if (st != ST_GROW) {
            return fail(st == ST_TABLE_FULL ? SQC_ERR_TABLE_FULL : SQC_ERR_STATE,
                        "device status " + std::to_string(st) + ": the state is no longer valid; reset it");
        }
        const size_t k = (size_t)(ctl_host_->seq - seq_verified_);
        if (k >= passes_.size()) return fail(SQC_ERR_STATE, "growth request outside a gate pass");
        if ((rc = repair(k))) return rc;
    }
    return fail(SQC_ERR_TABLE_FULL, "table growth did not converge");
}

// Copy the live, non-empty buckets into a new table of nb_new buckets. The control block
// must be in sync with the device (read_ctl) and no pass may be in flight.
int Engine::rebuild(unsigned long long nb_new) {
    HostTable nt;
    int rc;
    if ((rc = alloc_table(nb_new, &nt))) return rc;
    const unsigned long long n_old = ctl_host_->list_n;
    Ctl c = *ctl_host_;
    c.epoch = 1;   // a fresh table
    epochs_ = 1;
    c.status = 0;
    c.done = 0;
    c.seq = 0;
    c.list_n = 0;
    c.list_tail = 0;
    c.empty_groups = 0;
    c.acc_nnz = c.acc_empty = c.acc_upd = 0;
    c.work = 0;
    c.units_n = 0;
    std::memcpy(ctl_host_, &c, sizeof c);
    if ((rc = cuda(cudaMemcpyAsync(ctl_, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "H2D ctl")))
        return rc;
    TableDev nd;
    nd.hdr = nt.hdr; nd.keys = nt.keys; nd.amps = nt.amps; nd.list = nt.list; nd.units = nt.units;
    nd.mask = nt.nb - 1;
    if ((rc = cuda(launch_rehash(dev(), n_old, nd, 1u, dbl_ ? 16 : 8, ctl_, sms_, stream_), "rehash"))) return rc;
    ++launches_;
    if ((rc = read_ctl())) return rc;
    if (ctl_host_->status != ST_OK) {
        free_table(&nt);
        return fail(SQC_ERR_TABLE_FULL, "rebuild into the new table failed");
    }
    ctl_host_->list_n = ctl_host_->list_tail;
    if ((rc = cuda(cudaMemcpyAsync(&ctl_->list_n, &ctl_host_->list_n, sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, stream_), "H2D list_n")) ||
        (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
        return rc;
    free_table(&tab_);
    tab_ = nt;
    seq_verified_ = 0;
    list_hint_ = std::max<unsigned long long>(ctl_host_->list_n, 1);
    ++rebuilds_;
    return SQC_OK;
}

// Pass k refused to start because the table might overflow. Nothing of it ran; the state
// is the output of pass k-1. Grow the table and queue pass k's gates (and all later ones)
// again, from the planner state saved with pass k.
int Engine::repair(size_t k) {
    const PassRec pr = passes_[k];
    const unsigned long long groups = ctl_host_->list_n;
    unsigned long long nb = std::max(tab_.nb * 2, pow2_at_least((unsigned long long)std::ceil(4.0 * (double)groups / kMaxLoad)));
    // near the budget, take the largest table that still fits (the pass may refuse again)
    unsigned long long fit = tab_.nb;
    while ((double)(fit * 2) * bucket_bytes() <= (double)budget_) fit *= 2;
    if (nb > fit && fit > tab_.nb) nb = fit;
    int rc;
    if ((rc = rebuild(nb))) return rc;
    std::vector<sqc_gate> again(log_.begin() + (long)pr.log_begin, log_.end());
    replays_ += passes_.size() - k;
    passes_run_ -= passes_.size() - k;
    gates_applied_ -= again.size();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    plan_ = pr.snap;
    snap_plan_ = plan_;
    snap_log_ = 0;
    again.insert(again.end(), pending_.begin(), pending_.end());
    pending_.swap(again);
    return SQC_OK;
}

int Engine::take_unapplied(std::vector<sqc_gate>* rest) {
    int rc;
    if ((rc = read_ctl())) return rc;
    if (ctl_host_->status != ST_GROW) return fail(SQC_ERR_STATE, "no refused pass to take back");
    const size_t k = (size_t)(ctl_host_->seq - seq_verified_);
    if (k >= passes_.size()) return fail(SQC_ERR_STATE, "refused pass not found");
    const PassRec pr = passes_[k];
    rest->assign(log_.begin() + (long)pr.log_begin, log_.end());
    rest->insert(rest->end(), pending_.begin(), pending_.end());
    gates_applied_ -= log_.size() - pr.log_begin;
    passes_run_ -= passes_.size() - k;
    // every pass from k on returned without touching the state: clear the refusal
    ctl_host_->status = ST_OK;
    if ((rc = cuda(cudaMemcpyAsync(&ctl_->status, &ctl_host_->status, sizeof(unsigned int), cudaMemcpyHostToDevice,
                                   stream_), "H2D status")) ||
        (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
        return rc;
    plan_ = pr.snap;
    snap_plan_ = plan_;
    snap_log_ = 0;
    log_.clear();
    passes_.clear();
    pending_.clear();
    desc_used_ = 0;
    seq_verified_ = ctl_host_->seq;
    list_hint_ = std::max<unsigned long long>(ctl_host_->list_n, 1);
    err.clear();
    return SQC_OK;
}

int Engine::nnz(uint64_t* out) {
    int rc = sync();
    if (rc) return rc;
    *out = ctl_host_->nnz;
    return SQC_OK;
}

int Engine::ensure_sort(size_t n) {
    if (n <= sort_cap_) return SQC_OK;
    const size_t cap = std::max<size_t>(n, 1024);
    for (void* p : {(void*)sort_.keys_out, (void*)sort_.re_out, (void*)sort_.im_out, (void*)sort_.idx_in,
                    (void*)sort_.idx_out, (void*)sort_.cum, sort_.tmp})
        if (p) cudaFree(p);
    sort_ = SortBuffers();
    sort_cap_ = 0;
    const size_t tmp = sort_scratch_bytes(cap);
    int rc;
    if ((rc = cuda(cudaMalloc(&sort_.keys_out, cap * 8), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.re_out, cap * 8), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.im_out, cap * 8), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.idx_in, cap * 4), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.idx_out, cap * 4), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.cum, cap * 8), "cudaMalloc(sort)")) ||
        (rc = cuda(cudaMalloc(&sort_.tmp, tmp), "cudaMalloc(sort)")))
        return rc;
    sort_.tmp_bytes = tmp;
    sort_cap_ = cap;
    return SQC_OK;
}

// Work queued on the state's stream after this reuses the readout buffers only once the
// asynchronous readout's copy (if one is in flight) has read them.
int Engine::readout_buffers_free() {
    if (!async_pending_) return SQC_OK;
    return cuda(cudaStreamWaitEvent(stream_, ev_copied_, 0), "wait for the readout copy");
}

int Engine::get_state_async(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n) {
    if (!n || (cap && (!keys || !re || !im))) return fail(SQC_ERR_ARG, "null argument");
    // the copy engines write the arrays while the caller goes on: page-locked host memory only
    void* host_ptr[4] = {keys, re, im, n};
    for (int i = 0; i < 4; ++i) {
        if (!host_ptr[i]) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host_ptr[i]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            return fail(SQC_ERR_ARG, "asynchronous readout needs page-locked host arrays");
        }
    }
    int rc;
    // the queued gates go to the device first, so that they run while the previous
    // asynchronous readout's copy finishes; that readout then completes
    if ((rc = flush())) return rc;
    if ((rc = readout_wait())) return rc;
    if (!copy_stream_) {
        if ((rc = cuda(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "cudaStreamCreate")) ||
            (rc = cuda(cudaEventCreateWithFlags(&ev_gathered_, cudaEventDisableTiming), "event")) ||
            (rc = cuda(cudaEventCreateWithFlags(&ev_copied_, cudaEventDisableTiming), "event")) ||
            (rc = cuda(cudaMallocHost(&h_async_n_, sizeof(unsigned long long)), "cudaMallocHost")))
            return rc;
    }
    unsigned long long got = 0;
    if ((rc = readout_to_device(0, 0, false, &got, false))) return rc;   // gathered on the state's stream
    // a whole-state readout gathers exactly the present keys: the synchronized count says how
    // many bytes the copies move (the gathered count travels too and is checked on completion)
    const unsigned long long expect = ctl_host_->nnz;
    const unsigned long long m = std::min<unsigned long long>(expect, cap);
    if ((rc = cuda(cudaEventRecord(ev_gathered_, stream_), "event")) ||
        (rc = cuda(cudaStreamWaitEvent(copy_stream_, ev_gathered_, 0), "wait")) ||
        (rc = cuda(cudaMemcpyAsync(h_async_n_, &ctl_->out_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                   copy_stream_), "D2H count")) ||
        (rc = cuda(cudaMemcpyAsync(n, &ctl_->out_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                   copy_stream_), "D2H count")))
        return rc;
    if (m && ((rc = cuda(cudaMemcpyAsync(keys, d_rk_, m * 8, cudaMemcpyDeviceToHost, copy_stream_), "D2H keys")) ||
              (rc = cuda(cudaMemcpyAsync(re, d_rr_, m * 8, cudaMemcpyDeviceToHost, copy_stream_), "D2H re")) ||
              (rc = cuda(cudaMemcpyAsync(im, d_ri_, m * 8, cudaMemcpyDeviceToHost, copy_stream_), "D2H im"))))
        return rc;
    if ((rc = cuda(cudaEventRecord(ev_copied_, copy_stream_), "event"))) return rc;
    async_cap_ = cap;
    async_expect_ = expect;
    async_pending_ = true;
    return SQC_OK;
}

int Engine::readout_wait() {
    if (!async_pending_) return SQC_OK;
    int rc;
    if ((rc = cuda(cudaEventSynchronize(ev_copied_), "wait for the readout copy"))) return rc;
    async_pending_ = false;
    if (*h_async_n_ != async_expect_) return fail(SQC_ERR_STATE, "asynchronous readout: entry count changed");
    if (*h_async_n_ > async_cap_) return fail(SQC_ERR_CAPACITY, "output arrays too small");
    return SQC_OK;
}

// Compact the present keys with (actual & mask) == value into the device readout arrays
// (actual keys); *got receives their number (also when it exceeds the arrays).
int Engine::readout_to_device(uint64_t mask, uint64_t value, bool drop_negl, unsigned long long* got, bool wait) {
    int rc = sync();
    if (rc) return rc;
    if ((rc = ensure_readout(ctl_host_->nnz))) return rc;
    if ((rc = readout_buffers_free())) return rc;
    if ((rc = cuda(cudaMemsetAsync(&ctl_->out_count, 0, sizeof(unsigned long long), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_readout(dev(), ctl_, list_hint_, plan_.frame, dbl_, d_rk_, d_rr_, d_ri_, rcap_, drop_negl,
                                  prune_, sms_, stream_, mask, value ^ (plan_.frame & mask)),
                   "readout")))
        return rc;
    ++launches_;
    if (!wait) return SQC_OK;
    if ((rc = read_ctl())) return rc;
    *got = ctl_host_->out_count;
    return SQC_OK;
}

int Engine::get_state(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    return get_state_where(0, 0, keys, re, im, cap, n, flags);
}

int Engine::get_state_where(uint64_t mask, uint64_t value, uint64_t* keys, double* re, double* im, uint64_t cap,
                            uint64_t* n, uint32_t flags) {
    unsigned long long got = 0;
    int rc = readout_to_device(mask, value, (flags & SQC_READ_DROP_NEGLIGIBLE) != 0, &got);
    if (rc) return rc;
    if (n) *n = got;
    if (got > cap) return fail(SQC_ERR_CAPACITY, "output arrays too small");
    if (got && (!keys || !re || !im)) return fail(SQC_ERR_ARG, "null output array");
    if (!got) return SQC_OK;
    const unsigned long long* sk = d_rk_;
    const double* sr = d_rr_;
    const double* si = d_ri_;
    if ((flags & SQC_READ_SORTED) && got > 1) {   // key sort on the device
        if ((rc = ensure_sort(got))) return rc;
        sort_.keys_in = d_rk_;
        sort_.re_in = d_rr_;
        sort_.im_in = d_ri_;
        if ((rc = cuda(sort_entries(sort_, got, nq_, false, sms_, stream_), "sort"))) return rc;
        launches_ += 3;
        sk = sort_.keys_out;
        sr = sort_.re_out;
        si = sort_.im_out;
    }
    if ((rc = cuda(cudaMemcpyAsync(keys, sk, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H keys")) ||
        (rc = cuda(cudaMemcpyAsync(re, sr, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H re")) ||
        (rc = cuda(cudaMemcpyAsync(im, si, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H im")) ||
        (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
        return rc;
    return SQC_OK;
}

// Snapshot file: "SQCSNAP1", uint32 nq, uint32 precision, uint64 n, keys (sorted), re, im.
int Engine::save(const char* path) {
    uint64_t n = 0;
    int rc = nnz(&n);
    if (rc) return rc;
    std::vector<uint64_t> k(n);
    std::vector<double> r(n), i(n);
    if ((rc = get_state(k.data(), r.data(), i.data(), n, &n, SQC_READ_SORTED))) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(SQC_ERR_ARG, std::string("cannot open ") + path + " for writing");
    const char magic[8] = {'S', 'Q', 'C', 'S', 'N', 'A', 'P', '1'};
    const uint32_t hdr[2] = {nq_, dbl_ ? (uint32_t)SQC_FP64 : (uint32_t)SQC_FP32};
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(hdr, 4, 2, f) == 2 && std::fwrite(&n, 8, 1, f) == 1 &&
              std::fwrite(k.data(), 8, n, f) == n && std::fwrite(r.data(), 8, n, f) == n &&
              std::fwrite(i.data(), 8, n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SQC_OK : fail(SQC_ERR_ARG, std::string("write failed: ") + path);
}

int Engine::load(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SQC_ERR_ARG, std::string("cannot open ") + path);
    char magic[8];
    uint32_t hdr[2];
    uint64_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "SQCSNAP1", 8) == 0 &&
              std::fread(hdr, 4, 2, f) == 2 && std::fread(&n, 8, 1, f) == 1;
    if (ok && hdr[0] != nq_) {
        std::fclose(f);
        return fail(SQC_ERR_ARG, "snapshot qubit count differs from the state's");
    }
    std::vector<uint64_t> k;
    std::vector<double> r, i;
    if (ok) {
        k.resize(n);
        r.resize(n);
        i.resize(n);
        ok = std::fread(k.data(), 8, n, f) == n && std::fread(r.data(), 8, n, f) == n && std::fread(i.data(), 8, n, f) == n;
    }
    std::fclose(f);
    if (!ok) return fail(SQC_ERR_ARG, std::string("not a snapshot file or truncated: ") + path);
    return set_state(k.data(), r.data(), i.data(), n);
}

int Engine::probability(uint64_t mask, uint64_t value, double* p) {
    if (!p) return fail(SQC_ERR_ARG, "null output");
    int rc = sync();
    if (rc) return rc;
    if ((rc = cuda(cudaMemsetAsync(sums_, 0, sizeof(ExactSums), stream_), "memset")) ||
        (rc = cuda(launch_pattern_prob(dev(), ctl_, list_hint_, dbl_, mask, value ^ (plan_.frame & mask), sums_, sms_,
                                       stream_),
                   "probability")))
        return rc;
    ++launches_;
    if ((rc = read_sums())) return rc;
    *p = exact_sum_value(sums_host_->c[SUM_NORM]);
    return SQC_OK;
}

// Projective measurement of one qubit: outcome 1 iff u < p1 / norm, then the keys of the other
// outcome are removed and the rest renormalised; the measured bit becomes known to the planner.
int Engine::measure(uint32_t qubit, double u, int* outcome, double* p1) {
    if (qubit >= nq_) return fail(SQC_ERR_ARG, "qubit out of range");
    if (!(u >= 0.0 && u < 1.0)) return fail(SQC_ERR_ARG, "u must be in [0, 1)");
    double norm = 0.0, one = 0.0;
    int rc;
    if ((rc = norm2(&norm)) || (rc = probability(1ULL << qubit, 1ULL << qubit, &one))) return rc;
    if (!(norm > 0.0)) return fail(SQC_ERR_STATE, "measurement of an empty state");
    const double prob1 = one / norm;
    const int out = u < prob1 ? 1 : 0;
    const double kept = out ? one : norm - one;
    if (!(kept > 0.0)) return fail(SQC_ERR_STATE, "measurement outcome of probability zero");
    const unsigned long long bit = 1ULL << qubit;
    const unsigned long long val = out ? bit : 0ULL;
    if ((rc = cuda(launch_collapse(dev(), ctl_, list_hint_, dbl_, bit, val ^ (plan_.frame & bit), 1.0 / std::sqrt(kept),
                                   sms_, stream_),
                   "collapse")))
        return rc;
    launches_ += 2;
    if ((rc = read_ctl())) return rc;
    plan_.kmask |= bit;
    plan_.kval = (plan_.kval & ~bit) | val;
    snap_plan_ = plan_;
    if (outcome) *outcome = out;
    if (p1) *p1 = prob1;
    return SQC_OK;
}

int Engine::sample(uint64_t shots, uint64_t seed, uint64_t* keys) {
    if (shots && !keys) return fail(SQC_ERR_ARG, "null output array");
    unsigned long long got = 0;
    int rc = readout_to_device(0, 0, false, &got);
    if (rc) return rc;
    if (!shots) return SQC_OK;
    if (!got) return fail(SQC_ERR_STATE, "sampling an empty state");
    if ((rc = ensure_sort(got))) return rc;
    sort_.keys_in = d_rk_;
    sort_.re_in = d_rr_;
    sort_.im_in = d_ri_;
    if ((rc = cuda(sort_entries(sort_, got, nq_, true, sms_, stream_), "sort"))) return rc;
    unsigned long long* d_out = nullptr;
    if ((rc = cuda(cudaMallocAsync(&d_out, shots * 8, stream_), "cudaMallocAsync(samples)"))) return rc;
    rc = cuda(launch_sample(sort_.keys_out, sort_.cum, got, seed, shots, d_out, sms_, stream_), "sample");
    if (!rc) rc = cuda(cudaMemcpyAsync(keys, d_out, shots * 8, cudaMemcpyDeviceToHost, stream_), "D2H samples");
    cudaFreeAsync(d_out, stream_);
    if (!rc) rc = cuda(cudaStreamSynchronize(stream_), "sync");
    launches_ += 5;
    return rc;
}

int Engine::norm2(double* out) {
    int rc = sync();
    if (rc) return rc;
    if ((rc = cuda(cudaMemsetAsync(sums_, 0, sizeof(ExactSums), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_norm(dev(), ctl_, list_hint_, dbl_, sums_, sms_, stream_), "norm"))) return rc;
    ++launches_;
    if ((rc = read_sums())) return rc;
    *out = exact_sum_value(sums_host_->c[SUM_NORM]);
    return SQC_OK;
}

int Engine::compare(Engine& b, double* fidelity, double* max_abs_err) {
    int rc;
    if ((rc = b.sync())) return fail(rc, "compare: " + b.err);
    return compare_with(b.dev(), b.ctl_, b.list_hint_, b.dbl_, b.plan_.frame, b.nq_, b.device_, fidelity,
                        max_abs_err);
}

int Engine::compare_with(const TableDev& tb, const Ctl* cb, unsigned long long hint_b, bool dbl_b,
                         unsigned long long frame_b, uint32_t nq_b, int device_b, double* fidelity,
                         double* max_abs_err) {
    if (nq_b != nq_) return fail(SQC_ERR_ARG, "states differ in qubit count");
    if (device_b != device_) return fail(SQC_ERR_ARG, "states live on different devices");
    int rc;
    if ((rc = sync())) return rc;
    if ((rc = cuda(cudaMemsetAsync(sums_, 0, sizeof(ExactSums), stream_), "memset")) ||
        (rc = cuda(cudaMemsetAsync(&ctl_->acc_max, 0, sizeof(unsigned long long), stream_), "memset")))
        return rc;
    if ((rc = cuda(launch_compare(dev(), ctl_, list_hint_, dbl_, tb, cb, std::max<unsigned long long>(hint_b, 1),
                                  dbl_b, plan_.frame ^ frame_b, ctl_, sums_, sms_, stream_),
                   "compare")))
        return rc;
    launches_ += 3;
    if ((rc = read_sums())) return rc;
    if ((rc = read_ctl())) return rc;
    const double ore = exact_sum_value(sums_host_->c[SUM_ORE]), oim = exact_sum_value(sums_host_->c[SUM_OIM]);
    const double na = exact_sum_value(sums_host_->c[SUM_NA]);
    // |b|^2 over b's keys: those a shares and those it lacks, added exactly before rounding
    unsigned long long nbc[kSumChunks];
    for (int i = 0; i < kSumChunks; ++i) nbc[i] = sums_host_->c[SUM_NB][i] + sums_host_->c[SUM_NB_ONLY][i];
    const double nb = exact_sum_value(nbc);
    double mx;
    std::memcpy(&mx, &ctl_host_->acc_max, sizeof(double));
    *fidelity = (na > 0 && nb > 0) ? (ore * ore + oim * oim) / (na * nb) : 0.0;
    *max_abs_err = mx;
    return SQC_OK;
}

int Engine::stats(sqc_stats* out) {
    std::memset(out, 0, sizeof *out);
    out->gates_applied = gates_applied_;
    out->passes = passes_run_;
    out->kernel_launches = launches_;
    out->buckets = tab_.nb;
    out->table_bytes = (uint64_t)(tab_.nb * bucket_bytes());
    out->replays = replays_;
    out->amp_updates = (ctl_host_ ? ctl_host_->amp_updates : 0) + host_upd_;
    out->alg_bytes = ctl_host_ ? ctl_host_->alg_bytes : 0;
    out->alg_bytes_pair = ctl_host_ ? ctl_host_->alg_bytes_pair : 0;
    out->passes_pair = passes_pair_;
    out->pass_ns_pair = pass_ns_pair_;
    out->pass_ns_stream = pass_ns_stream_;
    return SQC_OK;
}

}  // namespace sqc
