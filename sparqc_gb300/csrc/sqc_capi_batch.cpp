// extern "C" entry points of the many-circuit batch and the serving loop (include/sparqc.h).
// Status codes only; no C++ exception crosses the boundary.
#include <new>
#include <string>

#include "../../include/sparqc.h"
#include "sqc_handles.h"

namespace {

template <class H, class F>
int guarded_impl(H& h, F&& f) {
    try {
        return f(h);
    } catch (const std::bad_alloc&) {
        h.err = "host allocation failed";
        return SQC_ERR_OOM;
    } catch (...) {
        h.err = "unexpected host exception";
        return SQC_ERR_STATE;
    }
}

template <class F>
int guarded(sqc_batch* bt, F&& f) {
    if (!bt) return SQC_ERR_ARG;
    return guarded_impl(bt->b, f);
}

template <class F>
int guarded(sqc_server* sv, F&& f) {
    if (!sv) return SQC_ERR_ARG;
    return guarded_impl(sv->s, f);
}

}  // namespace

extern "C" {

void sqc_batch_default_options(sqc_batch_options* opt) {
    if (!opt) return;
    opt->precision = SQC_FP64;
    opt->device = 0;
    opt->stream = nullptr;
    opt->prune_threshold = 1e-14;
    opt->load_factor = 0.45;
    opt->min_chunk = 8;
    opt->blocks_per_sm = 0;
    opt->memory_budget = 0;
    opt->use_graph = 0;
    opt->idle_limit_us = 0;
    opt->threads_per_unit = 0;
    opt->schedule_gates = 0;
    for (int i = 0; i < 2; ++i) opt->reserved[i] = 0;
}

int sqc_batch_create(const sqc_batch_options* opt, sqc_batch** out) {
    if (!out) return SQC_ERR_ARG;
    *out = nullptr;
    sqc_batch* bt = nullptr;
    try {
        bt = new sqc_batch();
    } catch (...) {
        return SQC_ERR_OOM;
    }
    int rc;
    try {
        rc = bt->b.init(opt);
    } catch (...) {
        rc = SQC_ERR_OOM;
    }
    if (rc != SQC_OK) {
        delete bt;
        return rc;
    }
    *out = bt;
    return SQC_OK;
}

int sqc_batch_destroy(sqc_batch* bt) {
    delete bt;
    return SQC_OK;
}

int sqc_batch_prepare(sqc_batch* bt, const sqc_circuit_desc* circuits, uint32_t n) {
    return guarded(bt, [&](sqc::Batch& b) { return b.prepare(circuits, n); });
}

int sqc_batch_run(sqc_batch* bt) { return guarded(bt, [](sqc::Batch& b) { return b.run(); }); }

int sqc_batch_sync(sqc_batch* bt) { return guarded(bt, [](sqc::Batch& b) { return b.sync(); }); }

int sqc_batch_circuit_status(sqc_batch* bt, uint32_t i, int* status) {
    return guarded(bt, [&](sqc::Batch& b) { return b.circuit_status(i, status); });
}

int sqc_batch_nnz(sqc_batch* bt, uint32_t i, uint64_t* nnz) {
    return guarded(bt, [&](sqc::Batch& b) { return b.nnz(i, nnz); });
}

int sqc_batch_get_state(sqc_batch* bt, uint32_t i, uint64_t* keys, double* re, double* im, uint64_t cap,
                        uint64_t* n, uint32_t flags) {
    return guarded(bt, [&](sqc::Batch& b) { return b.get_state(i, keys, re, im, cap, n, flags); });
}

int sqc_batch_get_states(sqc_batch* bt, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* counts,
                         uint64_t* total, uint32_t flags) {
    return guarded(bt, [&](sqc::Batch& b) { return b.get_states(keys, re, im, cap, counts, total, flags); });
}

int sqc_batch_autotune(sqc_batch* bt, sqc_batch_tuning* out) {
    return guarded(bt, [&](sqc::Batch& b) { return b.autotune(out); });
}

int sqc_batch_get_stats(sqc_batch* bt, sqc_batch_stats* out) {
    if (!out) return SQC_ERR_ARG;
    return guarded(bt, [&](sqc::Batch& b) { return b.stats(out); });
}

int sqc_batch_compare(sqc_batch* bt, uint32_t i, sqc_state* ref, double* fidelity, double* max_abs_err) {
    if (!ref || !fidelity || !max_abs_err) return SQC_ERR_ARG;
    return guarded(bt, [&](sqc::Batch& b) {
        sqc::TableDev t;
        const sqc::Ctl* c = nullptr;
        unsigned long long hint = 0, frame = 0;
        uint32_t nq = 0;
        bool dbl = true;
        int rc = b.table_of(i, &t, &c, &hint, &frame, &nq, &dbl);
        if (rc) return rc;
        rc = ref->eng.compare_with(t, c, hint, dbl, frame, nq, b.device(), fidelity, max_abs_err);
        if (rc) b.err = ref->eng.err;
        return rc;
    });
}

const char* sqc_batch_last_error(sqc_batch* bt) { return bt ? bt->b.err.c_str() : "null handle"; }

void* sqc_batch_stream(sqc_batch* bt) { return bt ? (void*)bt->b.stream() : nullptr; }

void sqc_server_default_options(sqc_server_options* opt) {
    if (!opt) return;
    opt->precision = SQC_FP64;
    opt->device = 0;
    opt->stream = nullptr;
    opt->prune_threshold = 1e-14;
    opt->load_factor = 0.45;
    opt->memory_budget = 0;
    opt->max_slots = 1024;
    opt->min_chunk = 8;
    opt->slice_ms = 2.0;
    opt->solo_log2_groups = 0;
    opt->solo_share_pct = 25;
    opt->inject_alloc_failures = 0;
    opt->schedule_gates = 0;
    opt->overlap_steps = 0;
    opt->reserved = 0;
}

int sqc_server_create(const sqc_server_options* opt, sqc_server** out) {
    if (!out) return SQC_ERR_ARG;
    *out = nullptr;
    sqc_server* sv = nullptr;
    try {
        sv = new sqc_server();
    } catch (...) {
        return SQC_ERR_OOM;
    }
    int rc;
    try {
        rc = sv->s.init(opt);
    } catch (...) {
        rc = SQC_ERR_OOM;
    }
    if (rc != SQC_OK) {
        delete sv;
        return rc;
    }
    *out = sv;
    return SQC_OK;
}

int sqc_server_destroy(sqc_server* sv) {
    delete sv;
    return SQC_OK;
}

int sqc_server_submit(sqc_server* sv, const sqc_circuit_desc* circuit, uint64_t* id) {
    return guarded(sv, [&](sqc::Server& s) { return s.submit(circuit, id); });
}

int sqc_server_step(sqc_server* sv, uint32_t* finished) {
    return guarded(sv, [&](sqc::Server& s) { return s.step(finished); });
}

int sqc_server_completed(sqc_server* sv, uint64_t* ids, uint32_t cap, uint32_t* n) {
    return guarded(sv, [&](sqc::Server& s) { return s.completed(ids, cap, n); });
}

int sqc_server_request_status(sqc_server* sv, uint64_t id, int* state, int* status) {
    return guarded(sv, [&](sqc::Server& s) { return s.request_status(id, state, status); });
}

int sqc_server_nnz(sqc_server* sv, uint64_t id, uint64_t* nnz) {
    return guarded(sv, [&](sqc::Server& s) { return s.nnz(id, nnz); });
}

int sqc_server_get_state(sqc_server* sv, uint64_t id, uint64_t* keys, double* re, double* im, uint64_t cap,
                         uint64_t* n, uint32_t flags) {
    return guarded(sv, [&](sqc::Server& s) { return s.get_state(id, keys, re, im, cap, n, flags); });
}

int sqc_server_release(sqc_server* sv, uint64_t id) {
    return guarded(sv, [&](sqc::Server& s) { return s.release(id); });
}

int sqc_server_get_stats(sqc_server* sv, sqc_server_stats* out) {
    if (!out) return SQC_ERR_ARG;
    return guarded(sv, [&](sqc::Server& s) { return s.stats(out); });
}

int sqc_server_compare(sqc_server* sv, uint64_t id, sqc_state* ref, double* fidelity, double* max_abs_err) {
    if (!ref || !fidelity || !max_abs_err) return SQC_ERR_ARG;
    return guarded(sv, [&](sqc::Server& s) {
        if (sqc::Engine* e = s.solo_engine(id)) {
            const int rc = ref->eng.compare(*e, fidelity, max_abs_err);
            if (rc) s.err = ref->eng.err;
            return rc;
        }
        sqc::TableDev t;
        const sqc::Ctl* c = nullptr;
        unsigned long long hint = 0, frame = 0;
        uint32_t nq = 0;
        bool dbl = true;
        int rc = s.table_of(id, &t, &c, &hint, &frame, &nq, &dbl);
        if (rc) return rc;
        rc = ref->eng.compare_with(t, c, hint, dbl, frame, nq, s.device(), fidelity, max_abs_err);
        if (rc) s.err = ref->eng.err;
        return rc;
    });
}

const char* sqc_server_last_error(sqc_server* sv) { return sv ? sv->s.err.c_str() : "null handle"; }

void* sqc_server_stream(sqc_server* sv) { return sv ? (void*)sv->s.stream() : nullptr; }

}  // extern "C"
