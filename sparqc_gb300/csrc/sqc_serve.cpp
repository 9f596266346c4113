// Serving loop: see sqc_serve.h.
#include "sqc_serve.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "sqc_kernels.h"

namespace sqc {

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr double kDefaultBudget = 120e9;   // bytes

}  // namespace

Server::~Server() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (void* p : {(void*)pool_, (void*)d_circ_, (void*)d_ctl_, (void*)d_sched_, (void*)d_words_, (void*)d_cmd_,
                    (void*)d_limit_, (void*)d_bctl_, (void*)d_rk_, (void*)d_rr_, (void*)d_ri_})
        if (p) cudaFree(p);
    for (void* p : {(void*)h_circ_, (void*)h_ctl_, (void*)h_sched_, (void*)h_cmd_, (void*)h_limit_, (void*)h_bctl_,
                    (void*)stg_circ_, (void*)stg_cmd_, (void*)stg_limit_})
        if (p) cudaFreeHost(p);
    reqs_.clear();   // solo engines release their tables before the stream goes
    spare_.clear();
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (ev2_) cudaEventDestroy(ev2_);
    for (cudaEvent_t e : solo_ev_) cudaEventDestroy(e);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

int Server::fail(int code, const std::string& msg) {
    err = msg;
    return code;
}

int Server::cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return SQC_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SQC_ERR_OOM : SQC_ERR_CUDA;
}

int Server::init(const sqc_server_options* opt) {
    sqc_server_options o;
    sqc_server_default_options(&o);
    if (opt) o = *opt;
    if (o.precision != SQC_FP64 && o.precision != SQC_FP32) return fail(SQC_ERR_ARG, "precision must be 32 or 64");
    if (!(o.prune_threshold > 0.0)) return fail(SQC_ERR_ARG, "prune_threshold must be > 0");
    if (!(o.load_factor > 0.0 && o.load_factor <= 0.45)) return fail(SQC_ERR_ARG, "load_factor must be in (0, 0.45]");
    if (o.min_chunk == 0 || (o.min_chunk & 3) || o.min_chunk > 4096) return fail(SQC_ERR_ARG, "bad min_chunk");
    if (o.max_slots == 0 || o.max_slots > (1u << 16)) return fail(SQC_ERR_ARG, "max_slots must be 1..65536");
    if (!(o.slice_ms > 0.0)) return fail(SQC_ERR_ARG, "slice_ms must be positive");
    if (o.solo_log2_groups > 64) return fail(SQC_ERR_ARG, "solo_log2_groups must be 0..64");
    if (o.solo_share_pct > 90) return fail(SQC_ERR_ARG, "solo_share_pct must be 0..90");
    dbl_ = o.precision == SQC_FP64;
    lf_ = o.load_factor;
    prune_thr_ = o.prune_threshold;
    const uint32_t sl = o.solo_log2_groups ? o.solo_log2_groups : 17;
    solo_min_groups_ = sl >= 64 ? ~0ULL : (1ULL << sl);
    min_chunk_ = o.min_chunk;
    max_slots_ = o.max_slots;
    slice_ms_ = o.slice_ms;
    inject_fail_ = o.inject_alloc_failures;
    sched_ = o.schedule_gates != 0;
    overlap_ = o.overlap_steps != 0;
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
    const size_t total_budget = o.memory_budget ? (size_t)o.memory_budget
                                                : (size_t)std::min(kDefaultBudget, 0.9 * (double)total_b);
    if (total_budget > free_b) return fail(SQC_ERR_BUDGET, "memory budget exceeds the free device memory");
    // the slice pool takes the budget but the share kept for solo circuits' own tables
    solo_cap_ = solo_min_groups_ == ~0ULL ? 0 : (size_t)((double)total_budget * o.solo_share_pct / 100.0);
    const size_t budget = total_budget - solo_cap_;
    if (o.stream) {
        stream_ = (cudaStream_t)o.stream;
    } else {
        if ((rc = cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
        own_stream_ = true;
    }
    const size_t n = max_slots_;
    if ((rc = cuda(cudaMalloc(&pool_, budget), "cudaMalloc(pool)")) ||
        (rc = cuda(cudaMalloc(&d_circ_, n * sizeof(BCirc)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_ctl_, n * sizeof(Ctl)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_sched_, n * sizeof(BSched)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_words_, n * sizeof(unsigned long long)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_cmd_, n * sizeof(unsigned)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_limit_, n * sizeof(unsigned)), "cudaMalloc")) ||
        (rc = cuda(cudaMalloc(&d_bctl_, sizeof(BatchCtl)), "cudaMalloc")) ||
        (rc = cuda(cudaMallocHost(&h_circ_, n * sizeof(BCirc)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&h_ctl_, n * sizeof(Ctl)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&h_sched_, n * sizeof(BSched)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&h_cmd_, n * sizeof(unsigned)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&h_limit_, n * sizeof(unsigned)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&h_bctl_, sizeof(BatchCtl)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&stg_circ_, n * sizeof(BCirc)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&stg_cmd_, n * sizeof(unsigned)), "cudaMallocHost")) ||
        (rc = cuda(cudaMallocHost(&stg_limit_, n * sizeof(unsigned)), "cudaMallocHost")) ||
        (rc = cuda(cudaMemset(d_ctl_, 0, n * sizeof(Ctl)), "cudaMemset")) ||
        (rc = cuda(cudaMemset(d_sched_, 0, n * sizeof(BSched)), "cudaMemset")) ||
        (rc = cuda(cudaMemset(d_words_, 0, n * sizeof(unsigned long long)), "cudaMemset")) ||
        (rc = cuda(cudaMemset(d_bctl_, 0, sizeof(BatchCtl)), "cudaMemset")) ||
        (rc = cuda(cudaEventCreate(&ev0_), "event")) || (rc = cuda(cudaEventCreate(&ev1_), "event")) ||
        (rc = cuda(cudaEventCreate(&ev2_), "event")))
        return rc;
    std::memset(h_circ_, 0, n * sizeof(BCirc));
    std::memset(h_cmd_, 0, n * sizeof(unsigned));
    std::memset(h_limit_, 0, n * sizeof(unsigned));
    alloc_.reset(budget);
    slot_req_.assign(n, 0);
    in_rid_.assign(n, 0);
    free_slots_.resize(n);
    for (size_t i = 0; i < n; ++i) free_slots_[i] = (int)(n - 1 - i);   // back() is the lowest slot
    return SQC_OK;
}

size_t Server::request_bytes(const Request& r) const {
    return slice_bytes(r.nb, dbl_) + align256(r.plan.desc.size() * sizeof(GateDesc)) +
           align256(r.plan.passes.size() * sizeof(BPass));
}

int Server::submit(const sqc_circuit_desc* c, uint64_t* id) {
    if (!c || !id) return fail(SQC_ERR_ARG, "null argument");
    Request r;
    if (const char* why = plan_circuit(c->nq, c->gates, c->n_gates, kMaxRun, 2, &r.plan)) return fail(SQC_ERR_ARG, why);
    r.nb = slice_buckets(r.plan.bound, lf_);
    r.solo = r.plan.bound >= solo_min_groups_ && r.nb && solo_bytes(r) <= solo_cap_;
    // schedule_gates order, for the passes that will run the circuit: the single-state engine's
    // (three cross-group qubits in FP32, two in FP64) or the pool's quads. The group bound, and
    // so the placement just decided, does not depend on the order.
    std::vector<sqc_gate> sched;
    if (sched_ && c->n_gates > 1 && c->n_gates <= kScheduleMaxGates) {
        std::vector<uint32_t> perm(c->n_gates);
        schedule_gates(c->gates, c->n_gates, r.solo && !dbl_ ? 3u : 2u, kMaxRun, kScheduleWindow, perm.data());
        sched.resize(c->n_gates);
        for (uint64_t j = 0; j < c->n_gates; ++j) sched[j] = c->gates[perm[j]];
        if (!r.solo) {
            r.plan = CircuitPlan();
            if (const char* why = plan_circuit(c->nq, sched.data(), sched.size(), kMaxRun, 2, &r.plan))
                return fail(SQC_ERR_ARG, why);
        }
    }
    if (r.solo) {
        if (sched.empty()) r.gates.assign(c->gates, c->gates + c->n_gates);
        else r.gates.swap(sched);
    } else if (!r.nb || request_bytes(r) > alloc_.size()) {
        return fail(SQC_ERR_BUDGET, "the circuit's table slice can never fit the memory budget");
    }
    const uint64_t rid = next_id_++;
    reqs_.emplace(rid, std::move(r));
    queue_.push_back(rid);
    *id = rid;
    return SQC_OK;
}

// Device bytes of a solo circuit's engine tables (sized so they never grow).
size_t Server::solo_bytes(const Request& r) const {
    const size_t per = sizeof(Header) + kSlots * 8 + kSlots * (dbl_ ? 16 : 8) + 4 + sizeof(Unit);
    return (size_t)r.nb * per;
}

int Server::admit_solo(uint64_t rid, Request& r) {
    if (inject_fail_) {   // testing aid: fail as an out-of-memory device would; nothing is held
        --inject_fail_;
        return fail(SQC_ERR_OOM, "injected allocation failure (large circuit's tables)");
    }
    for (size_t i = 0; i < spare_.size(); ++i) {   // a kept engine of the same shape: reset it
        if (spare_[i].nq != r.plan.nq || spare_[i].nb != r.nb) continue;
        std::unique_ptr<Engine> e = std::move(spare_[i].eng);
        solo_used_ -= spare_[i].bytes;
        spare_.erase(spare_.begin() + (std::ptrdiff_t)i);
        const int rc = e->set_zero();
        if (rc) {
            err = "solo engine: " + e->err;
            return rc;
        }
        r.eng = std::move(e);
        solo_used_ += solo_bytes(r);
        r.state = SQC_REQ_RUNNING;
        solo_.push_back(rid);
        return SQC_OK;
    }
    sqc_options o;
    sqc_default_options(&o);
    o.precision = dbl_ ? SQC_FP64 : SQC_FP32;
    o.prune_threshold = prune_thr_;
    o.initial_buckets = r.nb;
    o.stream = nullptr;   // its own stream: the large circuits' slices of a step run side by side
    o.device = (uint32_t)device_;
    sqc_hash_table_parameters hp;
    std::memset(&hp, 0, sizeof hp);
    hp.N_devices = 1;
    hp.coef_gpu_memory_reserve = 0.0;
    r.eng.reset(new Engine());
    int rc = r.eng->init(r.plan.nq, &hp, &o);
    if (rc) {
        err = "solo engine: " + r.eng->err;
        r.eng.reset();
        return rc;
    }
    solo_used_ += solo_bytes(r);
    r.state = SQC_REQ_RUNNING;
    solo_.push_back(rid);
    return SQC_OK;
}

// Admit queued requests in arrival order while a slot and pool memory are free (solo circuits:
// while the solo share of the budget has room).
int Server::admit() {
    int rc;
    while (!queue_.empty()) {
        const uint64_t rid = queue_.front();
        Request& r = reqs_.at(rid);
        if (r.solo) {
            // a spare engine of this shape is reused in place; others go when the room is needed
            size_t reuse = 0;
            for (const Spare& sp : spare_)
                if (sp.nq == r.plan.nq && sp.nb == r.nb) reuse = sp.bytes;
            while (solo_used_ - reuse + solo_bytes(r) > solo_cap_) {
                size_t k = 0;
                while (k < spare_.size() && spare_[k].nq == r.plan.nq && spare_[k].nb == r.nb) ++k;
                if (k == spare_.size()) break;
                solo_used_ -= spare_[k].bytes;
                spare_.erase(spare_.begin() + (std::ptrdiff_t)k);   // frees its tables
            }
            if (solo_used_ - reuse + solo_bytes(r) > solo_cap_) break;
            if ((rc = admit_solo(rid, r))) return rc;
            queue_.pop_front();
            continue;
        }
        if (free_slots_.empty()) break;
        if (inject_fail_) {   // testing aid: fail as an out-of-memory device would; the request stays queued
            --inject_fail_;
            return fail(SQC_ERR_OOM, "injected allocation failure (pool placement)");
        }
        const size_t bytes = request_bytes(r);
        const size_t off = alloc_.alloc(bytes);
        if (off == SIZE_MAX) break;
        std::sort(free_slots_.begin(), free_slots_.end(), std::greater<int>());
        const int slot = free_slots_.back();
        free_slots_.pop_back();
        r.slot = slot;
        r.off = off;
        r.bytes = bytes;
        unsigned char* base = pool_ + off;
        r.table = slice_table(base, r.nb, dbl_);
        GateDesc* dd = reinterpret_cast<GateDesc*>(base + slice_bytes(r.nb, dbl_));
        BPass* dp = reinterpret_cast<BPass*>(reinterpret_cast<unsigned char*>(dd) +
                                             align256(r.plan.desc.size() * sizeof(GateDesc)));
        if ((rc = cuda(cudaMemsetAsync(r.table.hdr, 0, r.nb * sizeof(Header), stream_), "cudaMemset(hdr)"))) return rc;
        if (!r.plan.desc.empty() &&
            (rc = cuda(cudaMemcpyAsync(dd, r.plan.desc.data(), r.plan.desc.size() * sizeof(GateDesc),
                                       cudaMemcpyHostToDevice, stream_), "H2D desc")))
            return rc;
        if (!r.plan.passes.empty() &&
            (rc = cuda(cudaMemcpyAsync(dp, r.plan.passes.data(), r.plan.passes.size() * sizeof(BPass),
                                       cudaMemcpyHostToDevice, stream_), "H2D passes")))
            return rc;
        BCirc& c = h_circ_[slot];
        std::memset(&c, 0, sizeof c);
        c.t = r.table;
        c.gates = dd;
        c.passes = dp;
        c.npasses = (uint32_t)r.plan.passes.size();
        c.max_groups = (unsigned long long)(0.9 * (double)r.nb);
        c.bound = r.plan.bound;
        h_cmd_[slot] = BC_INIT;
        h_limit_[slot] = c.npasses;
        r.state = SQC_REQ_RUNNING;
        slot_req_[slot] = rid;
        n_used_ = std::max<uint32_t>(n_used_, (uint32_t)slot + 1);
        queue_.pop_front();
    }
    return SQC_OK;
}

BatchArgs Server::args(uint32_t n) const {
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.circ = d_circ_;
    a.ctl = d_ctl_;
    a.sched = d_sched_;
    a.words = d_words_;
    a.bctl = d_bctl_;
    a.cmd = d_cmd_;
    a.limit = d_limit_;
    a.n = n;
    a.amp_bytes = dbl_ ? 16u : 8u;
    a.min_chunk = min_chunk_;
    const unsigned long long warps = (unsigned long long)sms_ * batch_residency(dbl_, 0) * 8;
    a.target_chunks = (uint32_t)std::min<unsigned long long>(kMaxChunks, 4 * warps);
    a.prune = prune_;
    a.idle_limit_ns = 2000000000ULL;   // a warp without work for 2 s ends the slice with ST_TIMEOUT
    return a;
}

int Server::step(uint32_t* finished) {
    if (finished) *finished = 0;
    int rc;
    uint32_t fin = 0;
    if (in_flight_) {
        // overlap_steps: the previous step's slice is still running. Admission (planning done,
        // engines made, slices cleared and uploaded) is host work and stream-ordered device
        // work, so it goes first; then the slice is retired. Retiring frees no memory, so
        // nothing more could be admitted after it.
        if ((rc = admit())) return rc;
        if ((rc = retire(&fin))) return rc;
        if (finished) *finished = fin;
    } else if ((rc = admit())) {
        return rc;
    }
    bool any = false;
    for (uint32_t s = 0; s < n_used_ && !any; ++s)
        any = slot_req_[s] && reqs_.at(slot_req_[s]).state == SQC_REQ_RUNNING;
    if (!any && solo_.empty()) return cuda(cudaStreamSynchronize(stream_), "sync");
    const uint32_t n = n_used_;
    if ((rc = cuda(cudaEventRecord(ev0_, stream_), "event"))) return rc;
    for (uint32_t s = 0; s < n; ++s)   // the requests this launch runs, for its retirement
        in_rid_[s] = slot_req_[s] && reqs_.at(slot_req_[s]).state == SQC_REQ_RUNNING ? slot_req_[s] : 0;
    if (any) {
        // the small circuits: one time slice of the persistent kernel over the resident slots
        std::memcpy(stg_circ_, h_circ_, n * sizeof(BCirc));
        std::memcpy(stg_cmd_, h_cmd_, n * sizeof(unsigned));
        std::memcpy(stg_limit_, h_limit_, n * sizeof(unsigned));
        if ((rc = cuda(cudaMemcpyAsync(d_circ_, stg_circ_, n * sizeof(BCirc), cudaMemcpyHostToDevice, stream_), "H2D")) ||
            (rc = cuda(cudaMemcpyAsync(d_cmd_, stg_cmd_, n * sizeof(unsigned), cudaMemcpyHostToDevice, stream_), "H2D")) ||
            (rc = cuda(cudaMemcpyAsync(d_limit_, stg_limit_, n * sizeof(unsigned), cudaMemcpyHostToDevice, stream_),
                       "H2D")))
            return rc;
        const int grid = sms_ * batch_residency(dbl_, 0);
        const unsigned long long slice_ns = (unsigned long long)(slice_ms_ * 1e6);
        if ((rc = cuda(launch_batch(args(n), dbl_, grid, 0, slice_ns, stream_), "batch launch")) ||
            (rc = cuda(cudaMemcpyAsync(h_sched_, d_sched_, n * sizeof(BSched), cudaMemcpyDeviceToHost, stream_), "D2H")) ||
            (rc = cuda(cudaMemcpyAsync(h_ctl_, d_ctl_, n * sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "D2H")) ||
            (rc = cuda(cudaMemcpyAsync(h_bctl_, d_bctl_, sizeof(BatchCtl), cudaMemcpyDeviceToHost, stream_), "D2H")))
            return rc;
        launches_ += 2;
    }
    if ((rc = cuda(cudaEventRecord(ev1_, stream_), "event"))) return rc;
    // the large circuits, after the batch slice, side by side on their engines' streams: each
    // applies as many of its next gates as fit a time slice at the rate the large circuits
    // together achieved on the previous steps (so a step holds about a slice per large circuit,
    // as when they ran one after the other); the server's stream then waits for all of them
    while (solo_ev_.size() < solo_.size()) {
        cudaEvent_t e;
        if ((rc = cuda(cudaEventCreate(&e), "event"))) return rc;
        solo_ev_.push_back(e);
    }
    for (size_t k = 0; k < solo_.size(); ++k) {
        Request& r = reqs_.at(solo_[k]);
        const cudaStream_t es = r.eng->stream();
        const uint64_t left = r.gates.size() - r.pos;
        uint64_t g = r.ms_per_gate > 0.0 ? (uint64_t)(slice_ms_ / r.ms_per_gate) : 32;
        g = std::min<uint64_t>(std::max<uint64_t>(8, g), left);
        r.chunk = g;
        if ((rc = cuda(cudaStreamWaitEvent(es, ev1_, 0), "wait"))) return rc;
        if (g && (rc = r.eng->apply(r.gates.data() + r.pos, g))) { err = r.eng->err; return rc; }
        // a slice that does not end the circuit keeps its last, unfinished pass queued, so the
        // pass goes on fusing the next slice's gates
        if ((rc = r.eng->flush(r.pos + g < r.gates.size()))) { err = r.eng->err; return rc; }
        if ((rc = cuda(cudaEventRecord(solo_ev_[k], es), "event")) ||
            (rc = cuda(cudaStreamWaitEvent(stream_, solo_ev_[k], 0), "wait")))
            return rc;
    }
    if ((rc = cuda(cudaEventRecord(ev2_, stream_), "event"))) return rc;
    in_flight_ = true;
    in_any_ = any;
    in_n_ = n;
    if (overlap_) return SQC_OK;
    rc = retire(&fin);
    if (finished) *finished += fin;
    return rc;
}

// Wait for the slice in flight and retire what it finished: solo circuits that applied their
// last gates, batch slots that ended (parked ones resume at the next launch).
int Server::retire(uint32_t* finished) {
    *finished = 0;
    in_flight_ = false;
    const bool any = in_any_;
    const uint32_t n = in_n_;
    int rc;
    if ((rc = cuda(cudaStreamSynchronize(stream_), "sync"))) return rc;
    ++steps_;
    float ms = 0.f, ms_solo = 0.f;
    if (cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) busy_ms_ += ms;
    if (cudaEventElapsedTime(&ms_solo, ev1_, ev2_) == cudaSuccess) busy_ms_ += ms_solo;
    uint32_t fin = 0;
    // solo circuits: measured rate (of all of them together), completion
    uint64_t solo_gates = 0;
    for (uint64_t rid : solo_) solo_gates += reqs_.at(rid).chunk;
    std::vector<uint64_t> still;
    for (uint64_t rid : solo_) {
        Request& r = reqs_.at(rid);
        if (solo_gates && ms_solo > 0.f) r.ms_per_gate = (double)ms_solo / (double)solo_gates;
        r.pos += r.chunk;
        r.chunk = 0;
        if (r.pos < r.gates.size()) {
            still.push_back(rid);
            continue;
        }
        rc = r.eng->sync();
        r.state = SQC_REQ_DONE;
        r.status = rc;
        if (rc == SQC_OK) {
            sqc_stats es;
            r.eng->stats(&es);
            r.amp_updates = es.amp_updates;
            upd_done_ += es.amp_updates;
            uint64_t nz = 0;
            r.eng->nnz(&nz);
            r.ctl.nnz = nz;
        }
        done_.push_back(rid);
        ++fin;
    }
    solo_.swap(still);
    // batch slots
    const bool timeout = any && h_bctl_->status == ST_TIMEOUT;
    for (uint32_t s = 0; any && s < n; ++s) {
        const uint64_t rid = slot_req_[s];
        if (!rid || rid != in_rid_[s]) continue;   // not run by this launch (free, done, or admitted since)
        Request& r = reqs_.at(rid);
        const unsigned st = h_sched_[s].state;
        if (st == BS_PARKED && !timeout) {
            h_cmd_[s] = BC_RESUME;
            continue;
        }
        h_cmd_[s] = BC_KEEP;
        r.state = SQC_REQ_DONE;
        r.ctl = h_ctl_[s];
        if (st == BS_DONE && r.ctl.status == ST_OK) {
            r.status = SQC_OK;
            upd_done_ += r.ctl.amp_updates + (uint64_t)r.plan.end.credit * r.ctl.nnz;
        } else {
            r.status = r.ctl.status == ST_TABLE_FULL ? SQC_ERR_TABLE_FULL : SQC_ERR_STATE;
        }
        done_.push_back(rid);
        ++fin;
    }
    *finished = fin;
    if (timeout) return fail(SQC_ERR_STATE, "serving kernel found no work for too long; running requests failed");
    return SQC_OK;
}

int Server::completed(uint64_t* ids, uint32_t cap, uint32_t* n) {
    if (!n || (cap && !ids)) return fail(SQC_ERR_ARG, "null argument");
    uint32_t k = 0;
    for (uint64_t id : done_) {
        if (k >= cap) break;
        ids[k++] = id;
    }
    *n = k;
    return SQC_OK;
}

int Server::request_status(uint64_t id, int* state, int* status) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(SQC_ERR_ARG, "unknown request");
    if (state) *state = it->second.state;
    if (status) *status = it->second.status;
    return SQC_OK;
}

int Server::nnz(uint64_t id, uint64_t* out) {
    auto it = reqs_.find(id);
    if (it == reqs_.end() || !out) return fail(SQC_ERR_ARG, "unknown request");
    if (it->second.state != SQC_REQ_DONE) return fail(SQC_ERR_STATE, "request not completed");
    *out = it->second.ctl.nnz;
    return SQC_OK;
}

Engine* Server::solo_engine(uint64_t id) {
    auto it = reqs_.find(id);
    return it != reqs_.end() && it->second.solo && it->second.state == SQC_REQ_DONE ? it->second.eng.get() : nullptr;
}

int Server::get_state(uint64_t id, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(SQC_ERR_ARG, "unknown request");
    Request& r = it->second;
    if (r.state != SQC_REQ_DONE) return fail(SQC_ERR_STATE, "request not completed");
    if (r.status != SQC_OK) return fail(r.status, "the request failed");
    int rc;
    if (r.solo) {
        rc = r.eng->get_state(keys, re, im, cap, n, flags);
        if (rc) err = r.eng->err;
        return rc;
    }
    const unsigned long long have = r.ctl.nnz;
    if (have > rcap_) {
        const size_t c = std::max<size_t>(have, 1024);
        for (void* p : {(void*)d_rk_, (void*)d_rr_, (void*)d_ri_}) if (p) cudaFree(p);
        d_rk_ = nullptr; d_rr_ = nullptr; d_ri_ = nullptr; rcap_ = 0;
        if ((rc = cuda(cudaMalloc(&d_rk_, c * 8), "cudaMalloc(readout)")) ||
            (rc = cuda(cudaMalloc(&d_rr_, c * 8), "cudaMalloc(readout)")) ||
            (rc = cuda(cudaMalloc(&d_ri_, c * 8), "cudaMalloc(readout)")))
            return rc;
        rcap_ = c;
    }
    Ctl* ctl = d_ctl_ + r.slot;
    if ((rc = cuda(cudaMemsetAsync(&ctl->out_count, 0, sizeof(unsigned long long), stream_), "memset"))) return rc;
    if ((rc = cuda(launch_readout(r.table, ctl, std::max<unsigned long long>(r.ctl.list_n, 1), r.plan.end.frame, dbl_,
                                  d_rk_, d_rr_, d_ri_, rcap_, (flags & SQC_READ_DROP_NEGLIGIBLE) != 0, prune_, sms_,
                                  stream_),
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

int Server::table_of(uint64_t id, TableDev* t, const Ctl** ctl, unsigned long long* hint, unsigned long long* frame,
                     uint32_t* nq, bool* dbl) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(SQC_ERR_ARG, "unknown request");
    const Request& r = it->second;
    if (r.state != SQC_REQ_DONE) return fail(SQC_ERR_STATE, "request not completed");
    if (r.status != SQC_OK) return fail(r.status, "the request failed");
    if (r.solo) return fail(SQC_ERR_STATE, "request ran on its own engine");
    *t = r.table;
    *ctl = d_ctl_ + r.slot;
    *hint = r.ctl.list_n;
    *frame = r.plan.end.frame;
    *nq = r.plan.nq;
    *dbl = dbl_;
    return SQC_OK;
}

int Server::release(uint64_t id) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(SQC_ERR_ARG, "unknown request");
    Request& r = it->second;
    if (r.state != SQC_REQ_DONE) return fail(SQC_ERR_STATE, "only completed requests can be released");
    if (r.solo) {
        if (r.eng && r.status == SQC_OK && spare_.size() < kMaxSpare) {
            // kept for the next large circuit of this shape; its bytes stay counted
            Spare sp;
            sp.eng = std::move(r.eng);
            sp.nq = r.plan.nq;
            sp.nb = r.nb;
            sp.bytes = solo_bytes(r);
            spare_.push_back(std::move(sp));
        } else {
            solo_used_ -= solo_bytes(r);
        }
        done_.erase(std::remove(done_.begin(), done_.end(), id), done_.end());
        reqs_.erase(it);   // an engine not kept frees its tables
        return SQC_OK;
    }
    const int slot = r.slot;
    alloc_.release(r.off, r.bytes);
    std::memset(&h_circ_[slot], 0, sizeof(BCirc));
    h_cmd_[slot] = BC_KEEP;
    h_limit_[slot] = 0;
    slot_req_[slot] = 0;
    free_slots_.push_back(slot);
    while (n_used_ > 0 && slot_req_[n_used_ - 1] == 0) --n_used_;
    done_.erase(std::remove(done_.begin(), done_.end(), id), done_.end());
    reqs_.erase(it);
    return SQC_OK;
}

int Server::stats(sqc_server_stats* out) {
    std::memset(out, 0, sizeof *out);
    out->queued = queue_.size();
    for (auto& kv : reqs_) out->running += kv.second.state == SQC_REQ_RUNNING ? 1 : 0;
    out->solo_running = solo_.size();
    out->completed = done_.size();
    out->steps = steps_;
    out->kernel_launches = launches_;
    out->amp_updates = upd_done_;
    out->pool_bytes = alloc_.size() + solo_cap_;
    size_t spare = 0;   // kept engines are reclaimable, not held by a request
    for (const Spare& sp : spare_) spare += sp.bytes;
    out->pool_used = alloc_.used() + solo_used_ - spare;
    out->busy_ms = busy_ms_;
    return SQC_OK;
}

}  // namespace sqc
