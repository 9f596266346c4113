// Partitioned state: a state that may outgrow the device (see sqc_part.h).
#include "sqc_part.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>

#include <cuda_runtime.h>

#include "sqc_plan.h"

namespace sqc {

namespace {

constexpr unsigned long long kLowBits = (1ULL << kSlotBits) - 1;   // qubits 0..3: inside a group
constexpr size_t kSample = 4096;                                   // keys sampled to balance splits
constexpr uint64_t kChunk = 1 << 20;                               // entries per host work item

bool non_diagonal(uint32_t kind) {
    return kind == SQC_X || kind == SQC_Y || kind == SQC_H || kind == SQC_RX || kind == SQC_RY || kind == SQC_U;
}

int popcount64(unsigned long long x) { return __builtin_popcountll(x); }

// Run f(item) for items [0, n) on up to `threads` threads (inline when there is one item).
template <class F>
void parallel_items(size_t n, int threads, F&& f) {
    const size_t nt = std::min<size_t>(n, (size_t)std::max(1, threads));
    if (nt <= 1) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (size_t t = 0; t < nt; ++t)
        pool.emplace_back([&, t]() {
            for (size_t i = t; i < n; i += nt) f(i);
        });
    for (std::thread& th : pool) th.join();
}

// Bin of key k under partition bits `bits` (bit j of the bin = bit bits[j] of the key).
inline size_t bin_of(uint64_t k, const std::vector<int>& bits) {
    size_t v = 0;
    for (size_t j = 0; j < bits.size(); ++j) v |= (size_t)((k >> bits[j]) & 1ULL) << j;
    return v;
}

// Largest partition a set of partition bits gives over a sample of keys.
size_t worst_bin(const std::vector<uint64_t>& sample, const std::vector<int>& bits) {
    std::vector<size_t> cnt(size_t(1) << bits.size(), 0);
    size_t worst = 0;
    for (uint64_t k : sample) worst = std::max(worst, ++cnt[bin_of(k, bits)]);
    return worst;
}

// Up to kSample keys spread evenly over the runs.
std::vector<uint64_t> sample_keys(const std::vector<const Run*>& runs) {
    uint64_t n = 0;
    for (const Run* r : runs) n += r->n;
    std::vector<uint64_t> s;
    if (!n) return s;
    const uint64_t step = std::max<uint64_t>(1, n / kSample);
    uint64_t at = 0;
    for (const Run* r : runs) {
        for (; at < r->n; at += step) s.push_back(r->k[at]);
        at -= r->n;
    }
    return s;
}

// Choose p bits of cand greedily, each time the one that keeps the largest sampled partition
// smallest.
std::vector<int> choose_bits(const std::vector<uint64_t>& sample, unsigned long long cand, int p) {
    std::vector<int> bits;
    for (int t = 0; t < p; ++t) {
        int best = -1;
        size_t best_w = ~size_t(0);
        for (int q = 0; q < 64; ++q) {
            if (!((cand >> q) & 1ULL)) continue;
            bits.push_back(q);
            const size_t w = worst_bin(sample, bits);
            bits.pop_back();
            if (w < best_w) { best_w = w; best = q; }
        }
        if (best < 0) break;
        bits.push_back(best);
        cand &= ~(1ULL << best);
    }
    return bits;
}

// A contiguous piece of a run, the unit of host work.
struct Piece {
    size_t run;
    uint64_t b, e;
};

std::vector<Piece> pieces_of(const std::vector<Run>& runs) {
    std::vector<Piece> ps;
    for (size_t r = 0; r < runs.size(); ++r)
        for (uint64_t b = 0; b < runs[r].n; b += kChunk) ps.push_back(Piece{r, b, std::min(runs[r].n, b + kChunk)});
    return ps;
}

}  // namespace

// ---- pinned pool and runs ----------------------------------------------------------------

PinnedPool::~PinnedPool() {
    for (auto& kv : blocks_) {
        if (kv.second.pinned) cudaFreeHost(kv.first);
        else std::free(kv.first);
    }
}

void* PinnedPool::get(size_t bytes) {
    bytes = std::max<size_t>(bytes, 64);
    auto it = free_.lower_bound(bytes);
    if (it != free_.end() && it->first <= 2 * bytes + (size_t(1) << 20)) {   // a cached block, not far too big
        void* p = it->second;
        free_.erase(it);
        return p;
    }
    const size_t cap = (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    void* p = nullptr;
    if (cudaMallocHost(&p, cap) == cudaSuccess && p) {
        blocks_[p] = Block{cap, true};
        return p;
    }
    cudaGetLastError();   // clear the failed pin
    while (!free_.empty()) {   // give cached blocks back before going to pageable memory
        auto f = free_.begin();
        if (blocks_[f->second].pinned) cudaFreeHost(f->second);
        else std::free(f->second);
        blocks_.erase(f->second);
        free_.erase(f);
    }
    if (cudaMallocHost(&p, cap) == cudaSuccess && p) {
        blocks_[p] = Block{cap, true};
        return p;
    }
    cudaGetLastError();
    p = std::malloc(cap);
    if (p) blocks_[p] = Block{cap, false};
    return p;
}

void PinnedPool::put(void* p) {
    auto it = blocks_.find(p);
    if (it != blocks_.end()) free_.emplace(it->second.bytes, p);
}

void Run::take(Run& o) {
    k = o.k; r = o.r; i = o.i; n = o.n;
    groups = o.groups; all_and = o.all_and; all_or = o.all_or;
    pool_ = o.pool_; block_ = o.block_;
    o.k = nullptr; o.r = nullptr; o.i = nullptr; o.n = 0;
    o.groups = 0; o.all_and = ~0ULL; o.all_or = 0;
    o.pool_ = nullptr; o.block_ = nullptr;
}

bool Run::alloc(PinnedPool* pool, uint64_t count) {
    release();
    void* b = pool->get((size_t)count * 24);
    if (!b) return false;
    pool_ = pool;
    block_ = b;
    k = static_cast<uint64_t*>(b);
    r = reinterpret_cast<double*>(k + count);
    i = r + count;
    n = count;
    return true;
}

void Run::release() {
    if (block_ && pool_) pool_->put(block_);
    block_ = nullptr;
    pool_ = nullptr;
    k = nullptr; r = nullptr; i = nullptr; n = 0;
    groups = 0; all_and = ~0ULL; all_or = 0;
}

void Run::fill_summary(int threads) {
    const size_t nc = (size_t)((n + kChunk - 1) / kChunk);
    std::vector<unsigned long long> a(nc, ~0ULL), o(nc, 0), g(nc, 0);
    parallel_items(nc, threads, [&](size_t c) {
        const uint64_t b = c * kChunk, e = std::min<uint64_t>(n, b + kChunk);
        unsigned long long aa = ~0ULL, oo = 0, gg = 0, prev = b ? (k[b - 1] >> kSlotBits) : ~0ULL;
        for (uint64_t x = b; x < e; ++x) {
            const unsigned long long key = k[x], grp = key >> kSlotBits;
            aa &= key;
            oo |= key;
            gg += grp != prev ? 1 : 0;
            prev = grp;
        }
        a[c] = aa; o[c] = oo; g[c] = gg;
    });
    all_and = ~0ULL;
    all_or = 0;
    groups = 0;
    for (size_t c = 0; c < nc; ++c) {
        all_and &= a[c];
        all_or |= o[c];
        groups += g[c];
    }
}

// ---- partitioned state -------------------------------------------------------------------

int PartState::fail(int code, const std::string& msg) {
    err = msg;
    return code;
}

int PartState::from_engine(int rc) {
    err = eng_.err;
    return rc;
}

int PartState::init(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt,
                    uint64_t device_bytes) {
    sqc_options o;
    sqc_default_options(&o);
    if (opt) o = *opt;
    if (device_bytes) {   // the first table within the cap too
        const uint64_t bucket = sizeof(Header) + kSlots * (8 + (o.precision == SQC_FP32 ? 8 : 16)) + sizeof(unsigned) +
                                sizeof(Unit);   // as the engine counts a bucket
        uint64_t nb = 64;
        while (nb < 1024 && (nb * 2) * bucket <= device_bytes) nb *= 2;
        if (!o.initial_buckets || o.initial_buckets > nb) o.initial_buckets = nb;
    }
    int rc = eng_.init(nq, params, &o);
    if (rc) return from_engine(rc);
    nq_ = nq;
    thr_ = o.prune_threshold;
    threads_ = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    eng_.limit_table_bytes((size_t)device_bytes);
    return SQC_OK;
}

void PartState::take_counters() {
    sqc_stats s;
    eng_.stats(&s);
    upd_ += s.amp_updates;
}

int PartState::set_zero() {
    take_counters();
    runs_.clear();
    pending_.clear();
    resident_ = true;
    const int rc = eng_.set_zero();
    return rc ? from_engine(rc) : SQC_OK;
}

int PartState::read_engine(Run* out) {
    uint64_t n = 0;
    int rc = eng_.nnz(&n);
    if (rc) return from_engine(rc);
    if (!out->alloc(&pool_, n)) return fail(SQC_ERR_OOM, "host memory for a partition");
    uint64_t got = 0;
    if ((rc = eng_.get_state(out->k, out->r, out->i, n, &got, 0))) return from_engine(rc);
    out->n = got;
    d2h_ += got * 24;
    out->fill_summary(threads_);
    return SQC_OK;
}

int PartState::load_engine(const Run& in) {
    take_counters();
    const Engine::KeySummary ks{in.all_and, in.all_or, in.groups};
    const int rc = eng_.set_state(in.k, in.r, in.i, in.n, &ks);
    if (rc) return from_engine(rc);
    h2d_ += in.n * 24;
    max_bin_ = std::max<uint64_t>(max_bin_, in.n);
    return SQC_OK;
}

// Keys one partition should start a window with: half of what the table budget holds at the
// growth load, at the state's keys per group.
uint64_t PartState::bin_keys_target() const {
    uint64_t n = 0, g = 0;
    for (const Run& r : runs_) {
        n += r.n;
        g += r.groups;
    }
    const double per_group = g ? std::min(16.0, std::max(1.0, (double)n / (double)g)) : 1.0;
    const double groups_cap = (double)eng_.table_budget() / (double)eng_.bucket_bytes_now() * 0.45;
    return (uint64_t)std::max(1.0, 0.5 * groups_cap * per_group);
}

// Move the entries of the runs into 2^|bits| bins by their partition bits, keeping their order
// (so each group stays contiguous): pieces of the runs are counted per bin in parallel, each
// piece gets its place in every bin, and the pieces are scattered in parallel. A bin's group
// count may count a group cut by a piece boundary twice (an upper bound, which only sizes the
// table). The runs are released.
int PartState::distribute(std::vector<Run>& runs, const std::vector<int>& bits, std::vector<Run>* bins) {
    const size_t nb = size_t(1) << bits.size();
    const std::vector<Piece> ps = pieces_of(runs);
    std::vector<uint64_t> cnt(ps.size() * nb, 0);
    parallel_items(ps.size(), threads_, [&](size_t c) {
        const Piece& p = ps[c];
        uint64_t* cc = &cnt[c * nb];
        const uint64_t* k = runs[p.run].k;
        for (uint64_t x = p.b; x < p.e; ++x) ++cc[bin_of(k[x], bits)];
    });
    bins->clear();
    bins->resize(nb);
    std::vector<uint64_t> off(ps.size() * nb);
    for (size_t v = 0; v < nb; ++v) {
        uint64_t at = 0;
        for (size_t c = 0; c < ps.size(); ++c) {
            off[c * nb + v] = at;
            at += cnt[c * nb + v];
        }
        if (at && !(*bins)[v].alloc(&pool_, at)) return fail(SQC_ERR_OOM, "host memory for a partition");
    }
    std::vector<unsigned long long> a(ps.size() * nb, ~0ULL), o(ps.size() * nb, 0), g(ps.size() * nb, 0);
    parallel_items(ps.size(), threads_, [&](size_t c) {
        const Piece& p = ps[c];
        const Run& src = runs[p.run];
        std::vector<unsigned long long> prev(nb, ~0ULL);
        for (uint64_t x = p.b; x < p.e; ++x) {
            const unsigned long long key = src.k[x];
            const size_t v = bin_of(key, bits);
            Run& d = (*bins)[v];
            const uint64_t at = off[c * nb + v]++;
            d.k[at] = key;
            d.r[at] = src.r[x];
            d.i[at] = src.i[x];
            const size_t s = c * nb + v;
            a[s] &= key;
            o[s] |= key;
            const unsigned long long grp = key >> kSlotBits;
            g[s] += grp != prev[v] ? 1 : 0;
            prev[v] = grp;
        }
    });
    for (size_t v = 0; v < nb; ++v) {
        Run& d = (*bins)[v];
        d.all_and = ~0ULL;
        d.all_or = 0;
        d.groups = 0;
        for (size_t c = 0; c < ps.size(); ++c) {
            d.all_and &= a[c * nb + v];
            d.all_or |= o[c * nb + v];
            d.groups += g[c * nb + v];
        }
    }
    for (Run& r : runs) r.release();
    return SQC_OK;
}

int PartState::apply(const sqc_gate* gates, uint64_t n) {
    if (n && !gates) return fail(SQC_ERR_ARG, "null gate array");
    if (resident_) {
        const int rc = eng_.apply(gates, n);
        if (rc == SQC_ERR_BUDGET) return sync();   // the table could not grow: spill and go on
        return rc ? from_engine(rc) : SQC_OK;
    }
    for (uint64_t i = 0; i < n; ++i) {
        if (const char* why = check_gate(gates[i], nq_)) return fail(SQC_ERR_ARG, why);
    }
    pending_.insert(pending_.end(), gates, gates + n);
    return SQC_OK;
}

// Run one partition through the device table with the given gates. A partition that does not
// fit, at the start or at a pass that could not grow the table, is split by one more bit of
// free_bits and each half continues with the gates that had not run.
int PartState::run_bin(Run& in, std::vector<sqc_gate> gates, unsigned long long free_bits, std::vector<Run>* out) {
    if (in.n == 0) return SQC_OK;
    int rc = load_engine(in);
    if (rc && rc != SQC_ERR_BUDGET) return rc;
    if (!rc) {
        in.release();
        if (!(rc = eng_.apply(gates.data(), gates.size()))) rc = eng_.sync();
        if (!rc) {
            Run res;
            if ((rc = read_engine(&res))) return rc;
            out->push_back(std::move(res));
            ++bins_;
            return SQC_OK;
        }
        if (rc != SQC_ERR_BUDGET) return from_engine(rc);
        std::vector<sqc_gate> rest;
        if ((rc = eng_.take_unapplied(&rest))) return from_engine(rc);
        if ((rc = read_engine(&in))) return rc;
        gates.swap(rest);
        ++bins_;
    }
    const unsigned long long cand = free_bits & (in.all_or ^ in.all_and) & ~kLowBits;
    if (!cand) return fail(SQC_ERR_BUDGET, "a partition outgrew the device budget and no qubit is left to split it by");
    const int b = choose_bits(sample_keys({&in}), cand, 1)[0];
    std::vector<Run> one;
    one.push_back(std::move(in));
    std::vector<Run> halves;
    if ((rc = distribute(one, {b}, &halves))) return rc;
    ++splits_;
    if ((rc = run_bin(halves[0], gates, free_bits & ~(1ULL << b), out))) return rc;
    return run_bin(halves[1], gates, free_bits & ~(1ULL << b), out);
}

// One window over the spilled state: partition bits, the gates they allow, every partition
// through the device.
int PartState::run_windows() {
    uint64_t n = 0;
    unsigned long long a = ~0ULL, o = 0;
    std::vector<const Run*> rp;
    for (const Run& r : runs_) {
        n += r.n;
        if (r.n) {
            a &= r.all_and;
            o |= r.all_or;
        }
        rp.push_back(&r);
    }
    if (n == 0) {   // no key can appear from an empty state
        pending_.clear();
        return SQC_OK;
    }
    // A window's partitions must start small enough for what its gates can add: a branching
    // gate on a qubit that is constant at the window's start can double a partition. p, the
    // number of partition qubits, follows from that bound. The window ends before the gate that
    // would leave fewer than p + 1 varying qubits untouched by its non-diagonal gates: p to
    // partition by and a spare one to split a partition that outgrows the device all the same
    // (the window's first gate may take the spare one).
    const double target = (double)bin_keys_target();
    const unsigned long long varying = (a ^ o) & ~kLowBits;
    auto bits_for = [&](int doublings) {
        int q = 0;
        while (q < 63 && std::ldexp((double)n, doublings - q) > target) ++q;
        return q;
    };
    size_t w = 0;
    unsigned long long touched = 0, grown = 0;
    int p = bits_for(0);
    for (; w < pending_.size(); ++w) {
        const sqc_gate& g = pending_[w];
        if (!non_diagonal(g.kind)) continue;
        const unsigned long long bit = 1ULL << g.target;
        const bool branching = g.kind != SQC_X && g.kind != SQC_Y;
        const unsigned long long t2 = touched | bit;
        const unsigned long long g2 = grown | (branching && !((a ^ o) & bit) ? bit : 0ULL);
        const int p2 = bits_for(popcount64(g2));
        if (popcount64(varying & ~t2) < p2 + (touched ? 1 : 0)) break;
        touched = t2;
        grown = g2;
        p = p2;
    }
    if (w == 0 || popcount64(varying & ~touched) < p)
        return fail(SQC_ERR_BUDGET, "the state is larger than the device budget and too few of its qubits vary to "
                                    "partition it around the next gate");
    const std::vector<int> bits = choose_bits(sample_keys(rp), varying & ~touched, p);
    std::vector<Run> bins;
    int rc = distribute(runs_, bits, &bins);
    runs_.clear();
    if (rc) return rc;
    unsigned long long pmask = 0;
    for (int q : bits) pmask |= 1ULL << q;
    const std::vector<sqc_gate> gates(pending_.begin(), pending_.begin() + (long)w);
    std::vector<Run> out;
    for (size_t v = 0; v < bins.size(); ++v) {
        if (!rc) rc = run_bin(bins[v], gates, varying & ~touched & ~pmask, &out);
        bins[v].release();
    }
    runs_.swap(out);
    if (rc) return rc;
    pending_.erase(pending_.begin(), pending_.begin() + (long)w);
    ++windows_;
    last_bits_ = (uint32_t)bits.size();
    return SQC_OK;
}

// Back to the device table when the whole state fits with room to grow.
int PartState::maybe_return() {
    uint64_t n = 0;
    for (const Run& r : runs_) n += r.n;
    if (n > bin_keys_target() / 2) return SQC_OK;
    Run all;
    if (!all.alloc(&pool_, n)) return fail(SQC_ERR_OOM, "host memory for the state");
    uint64_t at = 0;
    for (Run& r : runs_) {
        std::memcpy(all.k + at, r.k, r.n * 8);
        std::memcpy(all.r + at, r.r, r.n * 8);
        std::memcpy(all.i + at, r.i, r.n * 8);
        at += r.n;
    }
    all.fill_summary(threads_);
    const int rc = load_engine(all);
    if (rc == SQC_ERR_BUDGET) return SQC_OK;   // stays in host memory
    if (rc) return rc;
    runs_.clear();
    resident_ = true;
    ++returns_;
    return SQC_OK;
}

int PartState::sync() {
    for (;;) {
        int rc;
        if (resident_) {
            if (!pending_.empty()) {
                rc = eng_.apply(pending_.data(), pending_.size());
                pending_.clear();
                if (rc && rc != SQC_ERR_BUDGET) return from_engine(rc);
            }
            rc = eng_.sync();
            if (rc == SQC_OK) return SQC_OK;
            if (rc != SQC_ERR_BUDGET) return from_engine(rc);
            // the table could not grow: the state so far moves to host memory
            std::vector<sqc_gate> rest;
            if ((rc = eng_.take_unapplied(&rest))) return from_engine(rc);
            Run all;
            if ((rc = read_engine(&all))) return rc;
            runs_.clear();
            runs_.push_back(std::move(all));
            resident_ = false;
            ++spills_;
            pending_.swap(rest);
            continue;
        }
        if (pending_.empty()) return SQC_OK;
        if ((rc = run_windows())) return rc;
        if ((rc = maybe_return())) return rc;
    }
}

int PartState::nnz(uint64_t* out) {
    int rc = sync();
    if (rc) return rc;
    if (resident_) return (rc = eng_.nnz(out)) ? from_engine(rc) : SQC_OK;
    uint64_t n = 0;
    for (const Run& r : runs_) n += r.n;
    *out = n;
    return SQC_OK;
}

int PartState::get_state(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    int rc = sync();
    if (rc) return rc;
    if (resident_) return (rc = eng_.get_state(keys, re, im, cap, n, flags)) ? from_engine(rc) : SQC_OK;
    const bool drop = (flags & SQC_READ_DROP_NEGLIGIBLE) != 0;
    // the readout filter of the device (|re| < thr and |im| < thr, decided in FP64)
    auto keep = [&](double r, double i) { return !drop || !(std::fabs(r) < thr_ && std::fabs(i) < thr_); };
    uint64_t got = 0;
    for (const Run& r : runs_)
        for (uint64_t i = 0; i < r.n; ++i) got += keep(r.r[i], r.i[i]) ? 1 : 0;
    if (n) *n = got;
    if (got > cap) return fail(SQC_ERR_CAPACITY, "output arrays too small");
    if (got && (!keys || !re || !im)) return fail(SQC_ERR_ARG, "null output array");
    std::vector<std::pair<uint64_t, std::pair<uint32_t, uint64_t>>> at;   // (key, (run, index))
    at.reserve(got);
    for (uint32_t ri = 0; ri < runs_.size(); ++ri) {
        const Run& r = runs_[ri];
        for (uint64_t i = 0; i < r.n; ++i)
            if (keep(r.r[i], r.i[i])) at.push_back({r.k[i], {ri, i}});
    }
    if (flags & SQC_READ_SORTED)
        std::sort(at.begin(), at.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    for (uint64_t m = 0; m < at.size(); ++m) {
        const Run& r = runs_[at[m].second.first];
        const uint64_t i = at[m].second.second;
        keys[m] = r.k[i];
        re[m] = r.r[i];
        im[m] = r.i[i];
    }
    return SQC_OK;
}

int PartState::stats(sqc_part_stats* out) {
    std::memset(out, 0, sizeof *out);
    sqc_stats s;
    eng_.stats(&s);
    out->spilled = resident_ ? 0u : 1u;
    out->partition_bits = last_bits_;
    out->spills = spills_;
    out->returns = returns_;
    out->windows = windows_;
    out->bins = bins_;
    out->splits = splits_;
    out->bytes_h2d = h2d_;
    out->bytes_d2h = d2h_;
    out->amp_updates = upd_ + s.amp_updates;
    out->max_bin_keys = max_bin_;
    out->table_budget = eng_.table_budget();
    return SQC_OK;
}

}  // namespace sqc
