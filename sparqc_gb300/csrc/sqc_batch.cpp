// Host side of the many-circuit batch: planning, slice layout, launch, readout, autotuning.
// See sqc_batch.h.
#include "sqc_batch.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "sqc_kernels.h"

namespace sqc {

namespace {

constexpr unsigned long long kMinSliceBuckets = 16;
constexpr unsigned long long kMaxSliceBuckets = 1ULL << 31;   // list entries are 32-bit bucket indices
constexpr double kMaxBatchLoad = 0.45;                        // bound / buckets: 2 * bound <= 0.9 * buckets

unsigned long long pow2_at_least(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return p;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

size_t slice_bytes(unsigned long long nb, bool dbl) {
    return align256(nb * sizeof(Header)) + align256(nb * kSlots * 8) + align256(nb * kSlots * (dbl ? 16 : 8)) +
           align256(nb * 4);
}

TableDev slice_table(unsigned char* base, unsigned long long nb, bool dbl) {
    TableDev t;
    std::memset(&t, 0, sizeof t);
    size_t off = 0;
    t.hdr = reinterpret_cast<Header*>(base + off);
    off += align256(nb * sizeof(Header));
    t.keys = reinterpret_cast<unsigned long long*>(base + off);
    off += align256(nb * kSlots * 8);
    t.amps = base + off;
    off += align256(nb * kSlots * (dbl ? 16 : 8));
    t.list = reinterpret_cast<unsigned*>(base + off);
    t.mask = nb - 1;
    return t;
}

unsigned long long slice_buckets(unsigned long long bound, double lf) {
    const double want = std::ceil((double)bound / lf);
    if (want > (double)kMaxSliceBuckets) return 0;
    return std::max(kMinSliceBuckets, pow2_at_least((unsigned long long)want));
}

const char* plan_circuit(uint32_t nq, const sqc_gate* gates, uint64_t n, uint32_t max_run, uint32_t max_nx,
                         CircuitPlan* out) {
    if (nq < 1 || nq > 64) return "qubit count must be 1..64";
    if (n && !gates) return "null gate array";
    CircuitPlan& c = *out;
    c = CircuitPlan();
    c.nq = nq;
    c.n_gates = n;
    Planner p;
    p.kmask = ~0ULL;   // |0...0>: every bit known to be 0
    p.kval = 0;
    c.desc.reserve(n);
    for (uint64_t i = 0; i < n; ++i) {
        if (const char* why = check_gate(gates[i], nq)) return why;
        GateDesc d;
        if (!plan_gate(p, gates[i], &d)) continue;
        d.pad = p.credit;
        p.credit = 0;
        c.desc.push_back(d);
    }
    c.end = p;
    split_passes(c.desc.data(), c.desc.size(), max_run, max_nx,
                 [&](size_t g0, size_t g1, uint32_t nx, uint32_t q1, uint32_t q2, uint32_t, bool fixed) {
                     BPass b;
                     std::memset(&b, 0, sizeof b);
                     b.g0 = (uint32_t)g0;
                     b.g1 = (uint32_t)g1;
                     b.nx = (uint16_t)nx;
                     b.keys_fixed = fixed ? 1 : 0;
                     b.q1 = (uint8_t)(nx >= 1 ? q1 : 0xFF);
                     b.q2 = (uint8_t)(nx >= 2 ? q2 : 0xFF);
                     c.passes.push_back(b);
                     encode_pass(c.desc.data(), g0, g1, q1);
                 });
    if (c.passes.size() > kMaxBatchPasses) return "too many passes for a batch circuit";
    c.bound = group_bound(p, nq);
    return nullptr;
}

Batch::~Batch() {
    if (stream_) cudaStreamSynchronize(stream_);
    drop_graph();
    for (void* p : {(void*)pool_, (void*)d_desc_, (void*)d_pass_, (void*)d_circ_, (void*)d_ctl_, (void*)d_sched_,
                    (void*)d_words_, (void*)d_cmd_, (void*)d_limit_, (void*)d_bctl_, (void*)d_rk_, (void*)d_rr_, (void*)d_ri_})
        if (p) cudaFree(p);
    if (h_ctl_) cudaFreeHost(h_ctl_);
    if (h_bctl_) cudaFreeHost(h_bctl_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

int Batch::fail(int code, const std::string& msg) {
    err = msg;
    return code;
}

int Batch::cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return SQC_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SQC_ERR_OOM : SQC_ERR_CUDA;
}

int Batch::init(const sqc_batch_options* opt) {
    sqc_batch_options o;
    sqc_batch_default_options(&o);
    if (opt) o = *opt;
    if (o.precision != SQC_FP64 && o.precision != SQC_FP32) return fail(SQC_ERR_ARG, "precision must be 32 or 64");
    if (!(o.prune_threshold > 0.0)) return fail(SQC_ERR_ARG, "prune_threshold must be > 0");
    if (!(o.load_factor > 0.0 && o.load_factor <= kMaxBatchLoad)) return fail(SQC_ERR_ARG, "load_factor must be in (0, 0.45]");
    if (o.min_chunk == 0 || (o.min_chunk & 3) || o.min_chunk > 4096) return fail(SQC_ERR_ARG, "min_chunk must be a multiple of 4 in 4..4096");
    dbl_ = o.precision == SQC_FP64;
    lf_ = o.load_factor;
    min_chunk_ = o.min_chunk;
    blocks_per_sm_ = o.blocks_per_sm;
    idle_limit_ns_ = o.idle_limit_us ? 1000ULL * o.idle_limit_us : 2000000000ULL;
    if (o.threads_per_unit != 0 && o.threads_per_unit != 16 && o.threads_per_unit != 32)
        return fail(SQC_ERR_ARG, "threads_per_unit must be 0, 16 or 32");
    max_nx_ = o.threads_per_unit == 16 ? 1u : 2u;
    sched_ = o.schedule_gates != 0;
    use_graph_ = o.use_graph != 0;
    device_ = (int)o.device;
    std::memcpy(&prune_.d, &o.prune_threshold, sizeof(double));
    float tf = (float)o.prune_threshold;
    if ((double)tf >= o.prune_threshold && tf > 0.0f) tf = std::nextafter(tf, 0.0f);
    std::memcpy(&prune_.f, &tf, sizeof(float));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device_) return fail(SQC_ERR_NO_DEVICE, "no CUDA device");
    int rc;
    if ((rc = cuda(cudaSetDevice(device_), "cudaSetDevice"))) return rc;
    cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_);
    size_t free_b = 0, total_b = 0;
    if ((rc = cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"))) return rc;
    budget_ = o.memory_budget ? (size_t)o.memory_budget : (size_t)(0.98 * (double)total_b);
    if (o.stream) {
        stream_ = (cudaStream_t)o.stream;
    } else {
        if ((rc = cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
        own_stream_ = true;
    }
    if ((rc = cuda(cudaEventCreate(&ev0_), "event")) || (rc = cuda(cudaEventCreate(&ev1_), "event"))) return rc;
    if ((rc = cuda(cudaMalloc(&d_bctl_, sizeof(BatchCtl)), "cudaMalloc(bctl)"))) return rc;
    if ((rc = cuda(cudaMemset(d_bctl_, 0, sizeof(BatchCtl)), "cudaMemset"))) return rc;
    if ((rc = cuda(cudaMallocHost(&h_bctl_, sizeof(BatchCtl)), "cudaMallocHost"))) return rc;
    return SQC_OK;
}

void Batch::drop_graph() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    graph_exec_ = nullptr;
    graph_ = nullptr;
}

int Batch::prepare(const sqc_circuit_desc* cs, uint32_t n) {
    if (n && !cs) return fail(SQC_ERR_ARG, "null circuit array");
    std::vector<uint32_t> nqs(n);
    std::vector<std::vector<sqc_gate>> gates(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (cs[i].n_gates && !cs[i].gates) return fail(SQC_ERR_ARG, "circuit " + std::to_string(i) + ": null gates");
        nqs[i] = cs[i].nq;
        gates[i].assign(cs[i].gates, cs[i].gates + cs[i].n_gates);
        if (sched_ && cs[i].n_gates > 1 && cs[i].n_gates <= kScheduleMaxGates) {   // schedule_gates order for quads, whatever the tuning
            for (uint64_t j = 0; j < cs[i].n_gates; ++j)
                if (const char* why = check_gate(cs[i].gates[j], cs[i].nq))
                    return fail(SQC_ERR_ARG, "circuit " + std::to_string(i) + ": " + why);
            std::vector<uint32_t> perm(cs[i].n_gates);
            schedule_gates(cs[i].gates, cs[i].n_gates, 2, kMaxRun, kScheduleWindow, perm.data());
            for (uint64_t j = 0; j < cs[i].n_gates; ++j) gates[i][j] = cs[i].gates[perm[j]];
        }
    }
    nqs_.swap(nqs);
    gates_.swap(gates);
    return plan_and_upload();
}

// Plan the stored circuits with the current pass layout (max_nx_), upload descriptors and
// passes, and lay out the slices.
int Batch::plan_and_upload() {
    const uint32_t n = (uint32_t)gates_.size();
    int rc;
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    std::vector<CircuitPlan> plans(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (const char* why = plan_circuit(nqs_[i], gates_[i].data(), gates_[i].size(), kMaxRun, max_nx_, &plans[i]))
            return fail(SQC_ERR_ARG, "circuit " + std::to_string(i) + ": " + why);
    }
    plans_.swap(plans);
    ran_ = synced_ = false;
    // descriptors and passes, concatenated
    size_t nd = 0, np = 0;
    for (const CircuitPlan& c : plans_) { nd += c.desc.size(); np += c.passes.size(); }
    if (nd > desc_cap_) {
        if (d_desc_) cudaFree(d_desc_);
        d_desc_ = nullptr;
        desc_cap_ = 0;
        if ((rc = cuda(cudaMalloc(&d_desc_, std::max<size_t>(nd, 1) * sizeof(GateDesc)), "cudaMalloc(desc)"))) return rc;
        desc_cap_ = std::max<size_t>(nd, 1);
    }
    if (np > pass_cap_) {
        if (d_pass_) cudaFree(d_pass_);
        d_pass_ = nullptr;
        pass_cap_ = 0;
        if ((rc = cuda(cudaMalloc(&d_pass_, std::max<size_t>(np, 1) * sizeof(BPass)), "cudaMalloc(passes)"))) return rc;
        pass_cap_ = std::max<size_t>(np, 1);
    }
    if (n > circ_cap_) {
        for (void* p : {(void*)d_circ_, (void*)d_ctl_, (void*)d_sched_, (void*)d_words_, (void*)d_cmd_, (void*)d_limit_})
            if (p) cudaFree(p);
        if (h_ctl_) cudaFreeHost(h_ctl_);
        d_circ_ = nullptr; d_ctl_ = nullptr; d_sched_ = nullptr; d_words_ = nullptr; d_cmd_ = nullptr; d_limit_ = nullptr;
        h_ctl_ = nullptr;
        circ_cap_ = 0;
        if ((rc = cuda(cudaMalloc(&d_circ_, n * sizeof(BCirc)), "cudaMalloc")) ||
            (rc = cuda(cudaMalloc(&d_ctl_, n * sizeof(Ctl)), "cudaMalloc")) ||
            (rc = cuda(cudaMalloc(&d_sched_, n * sizeof(BSched)), "cudaMalloc")) ||
            (rc = cuda(cudaMalloc(&d_words_, n * sizeof(unsigned long long)), "cudaMalloc")) ||
            (rc = cuda(cudaMalloc(&d_cmd_, n * sizeof(unsigned)), "cudaMalloc")) ||
            (rc = cuda(cudaMalloc(&d_limit_, n * sizeof(unsigned)), "cudaMalloc")) ||
            (rc = cuda(cudaMallocHost(&h_ctl_, n * sizeof(Ctl)), "cudaMallocHost")))
            return rc;
        circ_cap_ = n;
    }
    if (n) {
        std::vector<GateDesc> hd;
        std::vector<BPass> hp;
        hd.reserve(nd);
        hp.reserve(np);
        for (const CircuitPlan& c : plans_) {
            hd.insert(hd.end(), c.desc.begin(), c.desc.end());
            hp.insert(hp.end(), c.passes.begin(), c.passes.end());
        }
        std::vector<unsigned> cmd(n, BC_INIT), lim(n);
        for (uint32_t i = 0; i < n; ++i) lim[i] = (unsigned)plans_[i].passes.size();
        if ((nd && (rc = cuda(cudaMemcpy(d_desc_, hd.data(), nd * sizeof(GateDesc), cudaMemcpyHostToDevice), "H2D"))) ||
            (np && (rc = cuda(cudaMemcpy(d_pass_, hp.data(), np * sizeof(BPass), cudaMemcpyHostToDevice), "H2D"))) ||
            (rc = cuda(cudaMemcpy(d_cmd_, cmd.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice), "H2D")) ||
            (rc = cuda(cudaMemcpy(d_limit_, lim.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice), "H2D")) ||
            (rc = cuda(cudaMemset(d_ctl_, 0, n * sizeof(Ctl)), "cudaMemset")) ||
            (rc = cuda(cudaMemset(d_sched_, 0, n * sizeof(BSched)), "cudaMemset")) ||
            (rc = cuda(cudaMemset(d_words_, 0, n * sizeof(unsigned long long)), "cudaMemset")))
            return rc;
    }
    return layout();
}

// Slice sizes from the group bounds and the load factor; one pool; the circuit array.
int Batch::layout() {
    drop_graph();
    ran_ = synced_ = false;
    const uint32_t n = (uint32_t)plans_.size();
    nb_.assign(n, 0);
    size_t total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        nb_[i] = slice_buckets(plans_[i].bound, lf_);
        if (!nb_[i])
            return fail(SQC_ERR_BUDGET, "circuit " + std::to_string(i) + ": its group bound needs more than 2^31 buckets");
        total += slice_bytes(nb_[i], dbl_);
    }
    const size_t fixed = desc_cap_ * sizeof(GateDesc) + pass_cap_ * sizeof(BPass) +
                         circ_cap_ * (sizeof(BCirc) + sizeof(Ctl) + sizeof(BSched) + 16);
    if (total + fixed > budget_) return fail(SQC_ERR_BUDGET, "the batch's table slices exceed the memory budget");
    int rc;
    if (total > pool_cap_) {
        if (pool_) cudaFree(pool_);
        pool_ = nullptr;
        pool_cap_ = 0;
        if ((rc = cuda(cudaMalloc(&pool_, total), "cudaMalloc(pool)"))) return rc;
        pool_cap_ = total;
    }
    pool_used_ = total;
    tables_.assign(n, TableDev());
    std::vector<BCirc> hc(n);
    size_t off = 0, doff = 0, poff = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const unsigned long long nb = nb_[i];
        TableDev& t = tables_[i];
        t = slice_table(pool_ + off, nb, dbl_);
        off += slice_bytes(nb, dbl_);
        // free every bucket of the slice (epoch 0 is never used)
        if ((rc = cuda(cudaMemsetAsync(t.hdr, 0, nb * sizeof(Header), stream_), "cudaMemset(hdr)"))) return rc;
        BCirc& c = hc[i];
        std::memset(&c, 0, sizeof c);
        c.t = t;
        c.gates = d_desc_ + doff;
        c.passes = d_pass_ + poff;
        c.npasses = (uint32_t)plans_[i].passes.size();
        c.max_groups = (unsigned long long)(0.9 * (double)nb);
        c.bound = plans_[i].bound;
        doff += plans_[i].desc.size();
        poff += plans_[i].passes.size();
    }
    if (n && (rc = cuda(cudaMemcpyAsync(d_circ_, hc.data(), n * sizeof(BCirc), cudaMemcpyHostToDevice, stream_), "H2D")))
        return rc;
    return cuda(cudaStreamSynchronize(stream_), "sync");
}

BatchArgs Batch::args() const {
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.circ = d_circ_;
    a.ctl = d_ctl_;
    a.sched = d_sched_;
    a.words = d_words_;
    a.bctl = d_bctl_;
    a.cmd = d_cmd_;
    a.limit = d_limit_;
    a.n = (uint32_t)plans_.size();
    a.amp_bytes = dbl_ ? 16u : 8u;
    a.min_chunk = min_chunk_;
    const unsigned long long warps = (unsigned long long)grid() * 8;
    a.target_chunks = (uint32_t)std::min<unsigned long long>(kMaxChunks, std::max<unsigned long long>(4 * warps, 1));
    a.prune = prune_;
    a.idle_limit_ns = idle_limit_ns_;
    return a;
}

int Batch::grid() const {
    const int res = batch_residency(dbl_, (int)blocks_per_sm_);
    const int per = blocks_per_sm_ ? std::min<int>((int)blocks_per_sm_, res) : res;
    return sms_ * std::max(per, 1);
}

int Batch::run() {
    if (plans_.empty()) return fail(SQC_ERR_STATE, "no circuits prepared");
    int rc;
    // every run restarts each circuit in a new epoch of its slice; before the 32-bit epoch could
    // come back round to a value still stored in a header, the headers are cleared (the run
    // restarts every circuit anyway) and the epoch starts over
    if (++epoch_runs_ >= kBatchEpochRestart) {
        for (const TableDev& t : tables_)
            if ((rc = cuda(cudaMemsetAsync(t.hdr, 0, (t.mask + 1) * sizeof(Header), stream_), "cudaMemset(hdr)")))
                return rc;
        if ((rc = cuda(cudaMemsetAsync(&d_bctl_->epoch, 0, sizeof(d_bctl_->epoch), stream_), "cudaMemset(epoch)")))
            return rc;
        epoch_runs_ = 1;
    }
    if ((rc = cuda(cudaEventRecord(ev0_, stream_), "event"))) return rc;
    if (use_graph_) {
        if (!graph_exec_) {
            if ((rc = cuda(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture"))) return rc;
            const cudaError_t le = launch_batch(args(), dbl_, grid(), (int)blocks_per_sm_, 0, stream_);
            const cudaError_t ce = cudaStreamEndCapture(stream_, &graph_);
            if ((rc = cuda(le, "batch launch (capture)")) || (rc = cuda(ce, "end capture"))) return rc;
            if ((rc = cuda(cudaGraphInstantiate(&graph_exec_, graph_, 0), "graph instantiate"))) return rc;
        }
        if ((rc = cuda(cudaGraphLaunch(graph_exec_, stream_), "graph launch"))) return rc;
    } else {
        if ((rc = cuda(launch_batch(args(), dbl_, grid(), (int)blocks_per_sm_, 0, stream_), "batch launch"))) return rc;
    }
    if ((rc = cuda(cudaEventRecord(ev1_, stream_), "event"))) return rc;
    launches_ += 2;
    ++runs_;
    ran_ = true;
    synced_ = false;
    return SQC_OK;
}

int Batch::read_ctl() {
    const size_t n = plans_.size();
    int rc;
    if (n && (rc = cuda(cudaMemcpyAsync(h_ctl_, d_ctl_, n * sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "D2H ctl")))
        return rc;
    if ((rc = cuda(cudaMemcpyAsync(h_bctl_, d_bctl_, sizeof(BatchCtl), cudaMemcpyDeviceToHost, stream_), "D2H bctl")))
        return rc;
    return cuda(cudaStreamSynchronize(stream_), "sync");
}

int Batch::sync() {
    if (!ran_) return fail(SQC_ERR_STATE, "the batch has not been run");
    int rc;
    if ((rc = read_ctl())) return rc;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) last_ms_ = ms;
    synced_ = true;
    if (h_bctl_->status == ST_TIMEOUT) return fail(SQC_ERR_STATE, "batch kernel found no work for too long");
    for (size_t i = 0; i < plans_.size(); ++i) {
        if (h_ctl_[i].status != ST_OK)
            return fail(SQC_ERR_STATE, "circuit " + std::to_string(i) + " failed with device status " +
                                           std::to_string(h_ctl_[i].status));
    }
    return SQC_OK;
}

int Batch::circuit_status(uint32_t i, int* status) {
    if (i >= plans_.size() || !status) return fail(SQC_ERR_ARG, "bad circuit index");
    if (!synced_) return fail(SQC_ERR_STATE, "sync the batch first");
    const unsigned s = h_ctl_[i].status;
    *status = s == ST_OK ? SQC_OK : s == ST_TABLE_FULL ? SQC_ERR_TABLE_FULL : SQC_ERR_STATE;
    return SQC_OK;
}

int Batch::nnz(uint32_t i, uint64_t* out) {
    if (i >= plans_.size() || !out) return fail(SQC_ERR_ARG, "bad circuit index");
    if (!synced_) return fail(SQC_ERR_STATE, "sync the batch first");
    *out = h_ctl_[i].nnz;
    return SQC_OK;
}

int Batch::ensure_readout(size_t n) {
    if (n <= rcap_) return SQC_OK;
    const size_t cap = std::max<size_t>(n, 1024);
    for (void* p : {(void*)d_rk_, (void*)d_rr_, (void*)d_ri_}) if (p) cudaFree(p);
    d_rk_ = nullptr; d_rr_ = nullptr; d_ri_ = nullptr; rcap_ = 0;
    int rc;
    if ((rc = cuda(cudaMalloc(&d_rk_, cap * 8), "cudaMalloc(readout)")) ||
        (rc = cuda(cudaMalloc(&d_rr_, cap * 8), "cudaMalloc(readout)")) ||
        (rc = cuda(cudaMalloc(&d_ri_, cap * 8), "cudaMalloc(readout)")))
        return rc;
    rcap_ = cap;
    return SQC_OK;
}

int Batch::get_states(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* counts, uint64_t* total,
                      uint32_t flags) {
    if (!synced_) return fail(SQC_ERR_STATE, "sync the batch first");
    const size_t nc = plans_.size();
    std::vector<unsigned long long> off(nc + 1, 0);
    for (size_t i = 0; i < nc; ++i) {
        if (h_ctl_[i].status != ST_OK) return fail(SQC_ERR_STATE, "circuit " + std::to_string(i) + " failed");
        off[i + 1] = off[i] + h_ctl_[i].nnz;
    }
    if (total) *total = off[nc];
    int rc;
    if ((rc = ensure_readout(off[nc]))) return rc;
    // circuit i's readout lands at offset off[i] (its key count bounds what it writes)
    for (size_t i = 0; i < nc; ++i) {
        Ctl* ctl = d_ctl_ + i;
        if ((rc = cuda(cudaMemsetAsync(&ctl->out_count, 0, sizeof(unsigned long long), stream_), "memset"))) return rc;
        if (!h_ctl_[i].nnz) continue;
        if ((rc = cuda(launch_readout(tables_[i], ctl, std::max<unsigned long long>(h_ctl_[i].list_n, 1),
                                      plans_[i].end.frame, dbl_, d_rk_ + off[i], d_rr_ + off[i], d_ri_ + off[i],
                                      h_ctl_[i].nnz, (flags & SQC_READ_DROP_NEGLIGIBLE) != 0, prune_, sms_, stream_),
                       "readout")))
            return rc;
        ++launches_;
    }
    if ((rc = cuda(cudaMemcpyAsync(h_ctl_, d_ctl_, nc * sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "D2H ctl")) ||
        (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
        return rc;
    uint64_t got = 0;
    for (size_t i = 0; i < nc; ++i) got += h_ctl_[i].out_count;
    if (total) *total = got;
    if (got > cap) return fail(SQC_ERR_CAPACITY, "output arrays too small");
    if (got && (!keys || !re || !im || !counts)) return fail(SQC_ERR_ARG, "null output array");
    if (!off[nc]) return SQC_OK;
    // without dropping, the circuits' entries are already contiguous: one copy per array
    const bool dense = got == off[nc];
    if (dense) {
        if ((rc = cuda(cudaMemcpyAsync(keys, d_rk_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H keys")) ||
            (rc = cuda(cudaMemcpyAsync(re, d_rr_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H re")) ||
            (rc = cuda(cudaMemcpyAsync(im, d_ri_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H im")))
            return rc;
    } else {
        uint64_t at = 0;
        for (size_t i = 0; i < nc; ++i) {
            const uint64_t c = h_ctl_[i].out_count;
            if (c && ((rc = cuda(cudaMemcpyAsync(keys + at, d_rk_ + off[i], c * 8, cudaMemcpyDeviceToHost, stream_),
                                 "D2H keys")) ||
                      (rc = cuda(cudaMemcpyAsync(re + at, d_rr_ + off[i], c * 8, cudaMemcpyDeviceToHost, stream_),
                                 "D2H re")) ||
                      (rc = cuda(cudaMemcpyAsync(im + at, d_ri_ + off[i], c * 8, cudaMemcpyDeviceToHost, stream_),
                                 "D2H im"))))
                return rc;
            at += c;
        }
    }
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    uint64_t at = 0;
    for (size_t i = 0; i < nc; ++i) {
        const uint64_t c = h_ctl_[i].out_count;
        counts[i] = c;
        if ((flags & SQC_READ_SORTED) && c > 1) {   // key order within each circuit
            std::vector<uint64_t> idx(c);
            std::iota(idx.begin(), idx.end(), 0);
            uint64_t* k = keys + at;
            double* r = re + at;
            double* im_ = im + at;
            std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return k[a] < k[b]; });
            std::vector<uint64_t> k2(c);
            std::vector<double> r2(c), i2(c);
            for (uint64_t j = 0; j < c; ++j) { k2[j] = k[idx[j]]; r2[j] = r[idx[j]]; i2[j] = im_[idx[j]]; }
            std::memcpy(k, k2.data(), c * 8);
            std::memcpy(r, r2.data(), c * 8);
            std::memcpy(im_, i2.data(), c * 8);
        }
        at += c;
    }
    return SQC_OK;
}

int Batch::get_state(uint32_t i, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    if (i >= plans_.size()) return fail(SQC_ERR_ARG, "bad circuit index");
    if (!synced_) return fail(SQC_ERR_STATE, "sync the batch first");
    if (h_ctl_[i].status != ST_OK) return fail(SQC_ERR_STATE, "the circuit failed");
    int rc;
    const unsigned long long have = h_ctl_[i].nnz;
    if ((rc = ensure_readout(have))) return rc;
    Ctl* ctl = d_ctl_ + i;
    if ((rc = cuda(cudaMemsetAsync(&ctl->out_count, 0, sizeof(unsigned long long), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_readout(tables_[i], ctl, std::max<unsigned long long>(h_ctl_[i].list_n, 1),
                                  plans_[i].end.frame, dbl_, d_rk_, d_rr_, d_ri_, rcap_,
                                  (flags & SQC_READ_DROP_NEGLIGIBLE) != 0, prune_, sms_, stream_),
                   "readout")))
        return rc;
    ++launches_;
    unsigned long long got = 0;
    if ((rc = cuda(cudaMemcpyAsync(&got, &ctl->out_count, sizeof got, cudaMemcpyDeviceToHost, stream_), "D2H")) ||
        (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
        return rc;
    if (n) *n = got;
    if (got > cap) return fail(SQC_ERR_CAPACITY, "output arrays too small");
    if (got && (!keys || !re || !im)) return fail(SQC_ERR_ARG, "null output array");
    if (got) {
        if ((rc = cuda(cudaMemcpyAsync(keys, d_rk_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H keys")) ||
            (rc = cuda(cudaMemcpyAsync(re, d_rr_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H re")) ||
            (rc = cuda(cudaMemcpyAsync(im, d_ri_, got * 8, cudaMemcpyDeviceToHost, stream_), "D2H im")) ||
            (rc = cuda(cudaStreamSynchronize(stream_), "sync")))
            return rc;
    }
    if ((flags & SQC_READ_SORTED) && got > 1) {
        std::vector<uint64_t> idx(got);
        std::iota(idx.begin(), idx.end(), 0);
        std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return keys[a] < keys[b]; });
        std::vector<uint64_t> k2(got);
        std::vector<double> r2(got), i2(got);
        for (uint64_t j = 0; j < got; ++j) { k2[j] = keys[idx[j]]; r2[j] = re[idx[j]]; i2[j] = im[idx[j]]; }
        std::memcpy(keys, k2.data(), got * 8);
        std::memcpy(re, r2.data(), got * 8);
        std::memcpy(im, i2.data(), got * 8);
    }
    return SQC_OK;
}

int Batch::table_of(uint32_t i, TableDev* t, const Ctl** ctl, unsigned long long* hint, unsigned long long* frame,
                    uint32_t* nq, bool* dbl) {
    if (i >= plans_.size()) return fail(SQC_ERR_ARG, "bad circuit index");
    if (!synced_) return fail(SQC_ERR_STATE, "sync the batch first");
    if (h_ctl_[i].status != ST_OK) return fail(SQC_ERR_STATE, "the circuit failed");
    *t = tables_[i];
    *ctl = d_ctl_ + i;
    *hint = h_ctl_[i].list_n;
    *frame = plans_[i].end.frame;
    *nq = plans_[i].nq;
    *dbl = dbl_;
    return SQC_OK;
}

int Batch::stats(sqc_batch_stats* out) {
    std::memset(out, 0, sizeof *out);
    out->circuits = plans_.size();
    out->table_bytes = pool_used_;
    out->kernel_launches = launches_;
    out->last_run_ms = last_ms_;
    if (synced_) {
        for (size_t i = 0; i < plans_.size(); ++i) {
            const Ctl& c = h_ctl_[i];
            out->passes += c.seq;
            out->amp_updates += c.amp_updates + (uint64_t)plans_[i].end.credit * c.nnz;
            out->alg_bytes += c.alg_bytes;
        }
    }
    return SQC_OK;
}

// Time each candidate tuning (two runs each, the faster counts) and keep the fastest. Threads
// per unit (pair or quad units: one or two qubits >= 4 per pass) changes the circuits' passes,
// the load factor the slice layout; chunk size and blocks per SM only the launch.
int Batch::autotune(sqc_batch_tuning* out) {
    if (plans_.empty()) return fail(SQC_ERR_STATE, "no circuits prepared");
    const double lf0 = lf_;
    const uint32_t ch0 = min_chunk_, bps0 = blocks_per_sm_, nx0 = max_nx_;
    int rc;
    auto time_it = [&](double* ms) -> int {
        double best = 1e300;
        for (int r = 0; r < 2; ++r) {
            int e;
            if ((e = run()) || (e = sync())) return e;
            best = std::min(best, last_ms_);
        }
        *ms = best;
        return SQC_OK;
    };
    double def_ms = 0;
    if ((rc = time_it(&def_ms))) return rc;
    double best_ms = def_ms, best_lf = lf0;
    uint32_t best_ch = ch0, best_bps = bps0, best_nx = nx0;
    uint32_t count = 1;
    const int res = std::max(batch_residency(dbl_, 0), batch_residency(dbl_, 2));
    for (uint32_t nx : {2u, 1u}) {
        if (nx != max_nx_) {
            max_nx_ = nx;
            if ((rc = plan_and_upload())) return rc;
        }
        for (double lf : {0.45, 0.25}) {
            lf_ = lf;
            if ((rc = layout())) {
                if (rc == SQC_ERR_BUDGET) continue;
                return rc;
            }
            for (uint32_t ch : {4u, 8u, 16u, 32u}) {
                for (int bps = 1; bps <= res; ++bps) {
                    min_chunk_ = ch;
                    blocks_per_sm_ = (uint32_t)bps;
                    drop_graph();
                    double ms = 0;
                    if ((rc = time_it(&ms))) return rc;
                    ++count;
                    if (ms < best_ms) {
                        best_ms = ms; best_lf = lf; best_ch = ch; best_bps = (uint32_t)bps; best_nx = nx;
                    }
                }
            }
        }
    }
    lf_ = best_lf;
    min_chunk_ = best_ch;
    blocks_per_sm_ = best_bps;
    if (best_nx != max_nx_) {
        max_nx_ = best_nx;
        if ((rc = plan_and_upload())) return rc;   // plans, uploads and lays out the slices
    } else if ((rc = layout())) {
        return rc;   // also drops a captured graph
    }
    if ((rc = run()) || (rc = sync())) return rc;
    if (out) {
        std::memset(out, 0, sizeof *out);
        out->load_factor = best_lf;
        out->min_chunk = best_ch;
        out->blocks_per_sm = best_bps;
        out->best_ms = best_ms;
        out->default_ms = def_ms;
        out->candidates = count;
        out->threads_per_unit = best_nx == 1 ? 16u : 32u;
    }
    return SQC_OK;
}

}  // namespace sqc
