// Host engine: table sizing and growth, pass planning, descriptor upload, deferred status
// checks with replay. See sqc_engine.h.
#include "sqc_engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "sqc_kernels.h"

namespace sqc {

namespace {

constexpr unsigned long long kMinBuckets = 64;
constexpr size_t kFlushAt = 1024;          // queued gates that trigger a launch
constexpr size_t kDescInitial = 1 << 14;   // descriptors held between verified syncs

unsigned long long pow2_at_least(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return p;
}

bool is_diag_kind(uint32_t k) {
    return k == SQC_Z || k == SQC_PHASE || k == SQC_RZ || k == SQC_S || k == SQC_SDG || k == SQC_T || k == SQC_TDG;
}
bool is_swap_kind(uint32_t k) { return k == SQC_X || k == SQC_Y; }

}  // namespace

Engine::~Engine() {
    if (stream_) cudaStreamSynchronize(stream_);
    free_tables(tab_);
    if (ctl_) cudaFree(ctl_);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    if (d_desc_) cudaFree(d_desc_);
    if (h_desc_) cudaFreeHost(h_desc_);
    if (d_rk_) cudaFree(d_rk_);
    if (d_rr_) cudaFree(d_rr_);
    if (d_ri_) cudaFree(d_ri_);
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

size_t Engine::bucket_bytes() const {
    return sizeof(Header) + kSlots * sizeof(unsigned long long) + kSlots * (dbl_ ? 16 : 8);
}

int Engine::init(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt) {
    sqc_options o;
    sqc_default_options(&o);
    if (opt) o = *opt;
    if (nq < 1 || nq > 64) return fail(SQC_ERR_ARG, "nq must be in 1..64");
    if (o.precision != SQC_FP64 && o.precision != SQC_FP32) return fail(SQC_ERR_ARG, "precision must be 64 or 32");
    if (!(o.prune_threshold > 0.0)) return fail(SQC_ERR_ARG, "prune_threshold must be > 0");
    if (!(o.load_factor > 0.0 && o.load_factor <= 0.9)) return fail(SQC_ERR_ARG, "load_factor must be in (0, 0.9]");
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

    prune_.d = 0;
    std::memcpy(&prune_.d, &thr_, sizeof(double));
    float tf = (float)thr_;
    if ((double)tf >= thr_) tf = std::nextafter(tf, 0.0f);
    std::memcpy(&prune_.f, &tf, sizeof(float));

    if ((rc = cuda(cudaMalloc(&ctl_, sizeof(Ctl)), "cudaMalloc(ctl)"))) return rc;
    if ((rc = cuda(cudaMemset(ctl_, 0, sizeof(Ctl)), "cudaMemset(ctl)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&ctl_host_, sizeof(Ctl)), "cudaMallocHost(ctl)"))) return rc;
    std::memset(ctl_host_, 0, sizeof(Ctl));
    if ((rc = ensure_desc(kDescInitial))) return rc;

    unsigned long long nb = pow2_at_least(std::max<unsigned long long>(o.initial_buckets ? o.initial_buckets : 1024, kMinBuckets));
    if ((rc = alloc_tables(nb, tab_))) return rc;
    return set_zero();
}

int Engine::alloc_tables(unsigned long long nb, HostTable out[2]) {
    if ((double)nb * bucket_bytes() * 2.0 > (double)budget_)
        return fail(SQC_ERR_BUDGET, "table memory would exceed the HBM budget");
    for (int i = 0; i < 2; ++i) {
        HostTable t;
        t.nb = nb;
        int rc;
        if ((rc = cuda(cudaMalloc(&t.hdr, nb * sizeof(Header)), "cudaMalloc(hdr)")) ||
            (rc = cuda(cudaMalloc(&t.keys, nb * kSlots * sizeof(unsigned long long)), "cudaMalloc(keys)")) ||
            (rc = cuda(cudaMalloc(&t.amps, nb * kSlots * (dbl_ ? 16 : 8)), "cudaMalloc(amps)")) ||
            (rc = cuda(cudaMemsetAsync(t.hdr, 0, nb * sizeof(Header), stream_), "cudaMemset(hdr)"))) {
            if (t.hdr) cudaFree(t.hdr);
            if (t.keys) cudaFree(t.keys);
            if (t.amps) cudaFree(t.amps);
            if (i == 1) free_tables(out);
            return rc;
        }
        out[i] = t;
    }
    return SQC_OK;
}

void Engine::free_tables(HostTable t[2]) {
    for (int i = 0; i < 2; ++i) {
        if (t[i].hdr) cudaFree(t[i].hdr);
        if (t[i].keys) cudaFree(t[i].keys);
        if (t[i].amps) cudaFree(t[i].amps);
        t[i] = HostTable();
    }
}

TableDev Engine::dev(const HostTable& t) const {
    TableDev d;
    d.hdr = t.hdr;
    d.keys = t.keys;
    d.amps = t.amps;
    d.mask = t.nb - 1;
    return d;
}

int Engine::ensure_desc(size_t n) {
    if (n <= desc_cap_) return SQC_OK;
    size_t cap = std::max(n, desc_cap_ * 2);
    if (d_desc_) cudaFree(d_desc_);
    if (h_desc_) cudaFreeHost(h_desc_);
    d_desc_ = nullptr;
    h_desc_ = nullptr;
    desc_cap_ = 0;
    int rc;
    if ((rc = cuda(cudaMalloc(&d_desc_, cap * sizeof(GateDesc)), "cudaMalloc(desc)"))) return rc;
    if ((rc = cuda(cudaMallocHost(&h_desc_, cap * sizeof(GateDesc)), "cudaMallocHost(desc)"))) return rc;
    desc_cap_ = cap;
    return SQC_OK;
}

int Engine::ensure_readout(size_t n) {
    if (n <= rcap_) return SQC_OK;
    size_t cap = std::max<size_t>(n, 1024);
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

GateDesc Engine::resolve(const sqc_gate& g) const {
    GateDesc d;
    std::memset(&d, 0, sizeof d);
    d.kind = g.kind;
    d.target = g.target;
    d.ctrl = g.controls;
    switch (g.kind) {
    case SQC_PHASE: d.c = std::cos(g.theta); d.s = std::sin(g.theta); break;
    case SQC_RZ: case SQC_RX: case SQC_RY: {
        const double h = g.theta / 2.;   // the reference passes par/2 (table_manager.cuh:333-336)
        d.c = std::cos(h);
        d.s = std::sin(h);
        break;
    }
    case SQC_T: d.c = 0.70710678118654752440; d.s = 0.70710678118654752440; break;
    case SQC_TDG: d.c = 0.70710678118654752440; d.s = -0.70710678118654752440; break;
    case SQC_H: d.c = 1. / std::sqrt(2.); break;   // as in h_core (device_data.cuh:205)
    case SQC_U: {
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

bool Engine::streamable(const sqc_gate& g) const {
    if (g.target < (uint32_t)kSlotBits) return true;
    if (is_diag_kind(g.kind)) return true;
    if (is_swap_kind(g.kind)) return (g.controls & 0xFULL) == 0;
    return false;
}

int Engine::set_zero() {
    pending_.clear();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    parity_ = 0;
    int rc = cuda(launch_set_zero(dev(tab_[0]), ctl_, 0, dbl_, stream_), "set_zero");
    ++launches_;
    return rc;
}

int Engine::set_state(const uint64_t* keys, const double* re, const double* im, uint64_t n) {
    if (n && (!keys || !re || !im)) return fail(SQC_ERR_ARG, "null array");
    for (uint64_t i = 0; i < n; ++i)
        if (nq_ < 64 && (keys[i] >> nq_)) return fail(SQC_ERR_ARG, "key does not fit in nq bits");
    int rc;
    // Wait for anything in flight, then size the tables for n keys in n groups at worst.
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    pending_.clear();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    unsigned long long need = pow2_at_least(std::max<unsigned long long>(kMinBuckets, (unsigned long long)std::ceil(n / lf_)));
    if (need > tab_[0].nb) {
        HostTable nt[2];
        if ((rc = alloc_tables(need, nt))) return rc;
        free_tables(tab_);
        tab_[0] = nt[0];
        tab_[1] = nt[1];
    }
    if ((rc = ensure_readout(n))) return rc;
    if (n) {
        if ((rc = cuda(cudaMemcpyAsync(d_rk_, keys, n * 8, cudaMemcpyHostToDevice, stream_), "H2D keys")) ||
            (rc = cuda(cudaMemcpyAsync(d_rr_, re, n * 8, cudaMemcpyHostToDevice, stream_), "H2D re")) ||
            (rc = cuda(cudaMemcpyAsync(d_ri_, im, n * 8, cudaMemcpyHostToDevice, stream_), "H2D im")))
            return rc;
    }
    parity_ = 0;
    if ((rc = cuda(cudaMemsetAsync(&ctl_->nnz[0], 0, sizeof(unsigned long long), stream_), "memset")) ||
        (rc = cuda(cudaMemsetAsync(&ctl_->groups[0], 0, sizeof(unsigned long long), stream_), "memset")))
        return rc;
    rc = cuda(launch_set_state(d_rk_, d_rr_, d_ri_, n, dev(tab_[0]), ctl_, 0, dbl_, sms_, stream_), "set_state");
    launches_ += n ? 5 : 3;
    if (rc) return rc;
    if ((rc = read_ctl())) return rc;
    if (ctl_host_->status == ST_DUPLICATE) {
        set_zero();
        return fail(SQC_ERR_ARG, "duplicate key in set_state");
    }
    if (ctl_host_->status != ST_OK) {
        set_zero();
        return fail(SQC_ERR_TABLE_FULL, "set_state: table full");
    }
    seq_verified_ = ctl_host_->seq;
    return SQC_OK;
}

int Engine::apply(const sqc_gate* gates, uint64_t n) {
    if (n && !gates) return fail(SQC_ERR_ARG, "null gate array");
    for (uint64_t i = 0; i < n; ++i) {
        const sqc_gate& g = gates[i];
        if (g.kind > SQC_U) return fail(SQC_ERR_ARG, "unknown gate kind");
        if (g.target >= nq_) return fail(SQC_ERR_ARG, "target qubit out of range");
        if (nq_ < 64 && (g.controls >> nq_)) return fail(SQC_ERR_ARG, "control qubit out of range");
        if ((g.controls >> g.target) & 1ULL) return fail(SQC_ERR_ARG, "target qubit among the controls");
    }
    pending_.insert(pending_.end(), gates, gates + n);
    if (pending_.size() >= kFlushAt) return flush();
    return SQC_OK;
}

PassArgs Engine::pass_args() const {
    PassArgs a;
    std::memset(&a, 0, sizeof a);
    a.tab[0] = dev(tab_[0]);
    a.tab[1] = dev(tab_[1]);
    a.ctl = ctl_;
    a.amp_bytes = dbl_ ? 16u : 8u;
    a.prune = prune_;
    return a;
}

// Split the queued gates into passes and launch them. A pass is either a run of streamable
// gates, or one cross-group gate followed by a run of streamable gates.
int Engine::flush() {
    if (pending_.empty()) return SQC_OK;
    const size_t n = pending_.size();
    int rc;
    if (desc_used_ + n > desc_cap_) {
        std::vector<sqc_gate> keep;
        keep.swap(pending_);
        if ((rc = sync())) return rc;          // verifies everything launched, resets desc_used_
        pending_.swap(keep);
        if ((rc = ensure_desc(n))) return rc;
    }
    GateDesc* hd = h_desc_ + desc_used_;
    for (size_t i = 0; i < n; ++i) hd[i] = resolve(pending_[i]);
    if ((rc = cuda(cudaMemcpyAsync(d_desc_ + desc_used_, hd, n * sizeof(GateDesc), cudaMemcpyHostToDevice, stream_),
                   "H2D gate descriptors")))
        return rc;
    const uint32_t log_base = (uint32_t)log_.size();
    log_.insert(log_.end(), pending_.begin(), pending_.end());
    PassArgs a = pass_args();
    a.gates = d_desc_ + desc_used_;
    size_t i = 0;
    while (i < n) {
        const size_t start = i;
        const bool pair = !streamable(pending_[i]);
        if (pair) ++i;
        while (i < n && i - start < max_run_ && streamable(pending_[i])) ++i;
        a.g0 = (uint32_t)start;
        a.g1 = (uint32_t)i;
        a.parity = (uint32_t)parity_;
        a.pair = pair ? 1u : 0u;
        bool fixed = true;
        for (size_t j = start; j < i; ++j) fixed = fixed && is_diag_kind(pending_[j].kind);
        a.keys_fixed = fixed ? 1u : 0u;
        if ((rc = cuda(launch_pass(a, dbl_, sms_, stream_), "gate pass"))) return rc;
        passes_.push_back(PassRec{log_base + (uint32_t)start, (uint32_t)(i - start), parity_, pair});
        parity_ ^= 1;
        ++launches_;
        ++passes_run_;
    }
    gates_applied_ += n;
    desc_used_ += n;
    pending_.clear();
    return SQC_OK;
}

int Engine::read_ctl() {
    int rc;
    if ((rc = cuda(cudaMemcpyAsync(ctl_host_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "D2H ctl")))
        return rc;
    return cuda(cudaStreamSynchronize(stream_), "sync");
}

int Engine::sync() {
    int rc;
    for (int attempt = 0; attempt < 64; ++attempt) {
        if ((rc = flush())) return rc;
        if ((rc = read_ctl())) return rc;
        if (ctl_host_->status == ST_OK) {
            seq_verified_ = ctl_host_->seq;
            log_.clear();
            passes_.clear();
            desc_used_ = 0;
            return SQC_OK;
        }
        if (ctl_host_->status != ST_TABLE_FULL) return fail(SQC_ERR_STATE, "device status error");
        const size_t k = (size_t)(ctl_host_->seq - seq_verified_);
        if (k >= passes_.size()) return fail(SQC_ERR_STATE, "table full outside a gate pass");
        if ((rc = repair(k))) return rc;
    }
    return fail(SQC_ERR_TABLE_FULL, "table growth did not converge");
}

// Pass k ran out of table space. Its input table is intact: move it into larger tables and
// queue the gates of pass k and of every later pass again.
int Engine::repair(size_t k) {
    const PassRec pr = passes_[k];
    const int pin = pr.parity_in;
    const unsigned long long groups_in = ctl_host_->groups[pin];
    unsigned long long nb = tab_[0].nb * 2;
    nb = std::max(nb, pow2_at_least((unsigned long long)std::ceil(2.0 * (double)groups_in / lf_)));
    HostTable nt[2];
    int rc;
    if ((rc = alloc_tables(nb, nt))) return rc;
    Ctl c = *ctl_host_;
    const unsigned ep_old = c.epoch[pin];
    std::memset(&c, 0, sizeof c);
    c.epoch[0] = 1;
    c.epoch[1] = 0;
    c.nnz[0] = ctl_host_->nnz[pin];
    c.groups[0] = ctl_host_->groups[pin];
    c.amp_updates = ctl_host_->amp_updates;
    c.alg_bytes = ctl_host_->alg_bytes;
    std::memcpy(ctl_host_, &c, sizeof c);
    if ((rc = cuda(cudaMemcpyAsync(ctl_, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "H2D ctl")))
        return rc;
    if ((rc = cuda(launch_rehash(dev(tab_[pin]), ep_old, dev(nt[0]), 1u, dbl_ ? 16 : 8, ctl_, sms_, stream_),
                   "rehash")))
        return rc;
    ++launches_;
    if ((rc = read_ctl())) return rc;
    if (ctl_host_->status != ST_OK) {
        free_tables(nt);
        return fail(SQC_ERR_TABLE_FULL, "rehash into the grown table failed");
    }
    free_tables(tab_);
    tab_[0] = nt[0];
    tab_[1] = nt[1];
    parity_ = 0;
    std::vector<sqc_gate> again(log_.begin() + pr.first_gate, log_.end());
    replays_ += passes_.size() - k;
    passes_run_ -= passes_.size() - k;
    gates_applied_ -= again.size();
    log_.clear();
    passes_.clear();
    seq_verified_ = 0;
    desc_used_ = 0;
    again.insert(again.end(), pending_.begin(), pending_.end());
    pending_.swap(again);
    return SQC_OK;
}

int Engine::nnz(uint64_t* out) {
    int rc = sync();
    if (rc) return rc;
    *out = ctl_host_->nnz[parity_];
    return SQC_OK;
}

int Engine::get_state(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    int rc = sync();
    if (rc) return rc;
    const unsigned long long have = ctl_host_->nnz[parity_];
    if ((rc = ensure_readout(have))) return rc;
    if ((rc = cuda(cudaMemsetAsync(&ctl_->out_count, 0, sizeof(unsigned long long), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_readout(dev(tab_[parity_]), ctl_, parity_, dbl_, d_rk_, d_rr_, d_ri_, rcap_,
                                  (flags & SQC_READ_DROP_NEGLIGIBLE) != 0, prune_, sms_, stream_),
                   "readout")))
        return rc;
    ++launches_;
    if ((rc = read_ctl())) return rc;
    const unsigned long long got = ctl_host_->out_count;
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
        for (uint64_t i = 0; i < got; ++i) { k2[i] = keys[idx[i]]; r2[i] = re[idx[i]]; i2[i] = im[idx[i]]; }
        std::memcpy(keys, k2.data(), got * 8);
        std::memcpy(re, r2.data(), got * 8);
        std::memcpy(im, i2.data(), got * 8);
    }
    return SQC_OK;
}

int Engine::norm2(double* out) {
    int rc = sync();
    if (rc) return rc;
    if ((rc = cuda(cudaMemsetAsync(&ctl_->acc[0], 0, sizeof(double), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_norm(dev(tab_[parity_]), ctl_, parity_, dbl_, sms_, stream_), "norm"))) return rc;
    ++launches_;
    if ((rc = read_ctl())) return rc;
    *out = ctl_host_->acc[0];
    return SQC_OK;
}

int Engine::compare(Engine& b, double* fidelity, double* max_abs_err) {
    if (b.nq_ != nq_) return fail(SQC_ERR_ARG, "states differ in qubit count");
    int rc;
    if ((rc = b.sync())) return fail(rc, "compare: " + b.err);
    if ((rc = sync())) return rc;
    if ((rc = cuda(cudaMemsetAsync(ctl_->acc, 0, sizeof(ctl_->acc), stream_), "memset")) ||
        (rc = cuda(cudaMemsetAsync(&ctl_->acc_max, 0, sizeof(unsigned long long), stream_), "memset")))
        return rc;
    if ((rc = cuda(launch_compare(dev(tab_[parity_]), ctl_host_->epoch[parity_], dbl_, b.dev(b.tab_[b.parity_]),
                                  b.ctl_host_->epoch[b.parity_], b.dbl_, ctl_, sms_, stream_),
                   "compare")))
        return rc;
    launches_ += 2;
    if ((rc = read_ctl())) return rc;
    const double ore = ctl_host_->acc[0], oim = ctl_host_->acc[1], na = ctl_host_->acc[2];
    const double nb = ctl_host_->acc[3] + ctl_host_->acc[4];
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
    out->buckets = tab_[0].nb;
    out->table_bytes = (uint64_t)(tab_[0].nb * bucket_bytes() * 2);
    out->replays = replays_;
    out->amp_updates = ctl_host_ ? ctl_host_->amp_updates : 0;
    out->alg_bytes = ctl_host_ ? ctl_host_->alg_bytes : 0;
    return SQC_OK;
}

}  // namespace sqc
