// extern "C" entry points of the partitioned state (include/sparqc.h, "states larger than the
// device budget"). Same conventions as the single-state entry points: status codes, no C++
// exception across the boundary.
#include <new>
#include <string>

#include "../../include/sparqc.h"
#include "sqc_handles.h"

namespace {

template <class F>
int guarded(sqc_part_state* st, F&& f) {
    if (!st) return SQC_ERR_ARG;
    try {
        return f(st->p);
    } catch (const std::bad_alloc&) {
        st->p.err = "host allocation failed";
        return SQC_ERR_OOM;
    } catch (...) {
        st->p.err = "unexpected host exception";
        return SQC_ERR_STATE;
    }
}

}  // namespace

extern "C" {

int sqc_part_create(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt,
                    uint64_t device_bytes, sqc_part_state** out) {
    if (!out) return SQC_ERR_ARG;
    *out = nullptr;
    sqc_part_state* st = nullptr;
    try {
        st = new sqc_part_state();
    } catch (...) {
        return SQC_ERR_OOM;
    }
    int rc;
    try {
        rc = st->p.init(nq, params, opt, device_bytes);
    } catch (...) {
        rc = SQC_ERR_OOM;
    }
    if (rc != SQC_OK) {
        delete st;
        return rc;
    }
    *out = st;
    return SQC_OK;
}

int sqc_part_destroy(sqc_part_state* st) {
    delete st;
    return SQC_OK;
}

int sqc_part_set_zero_state(sqc_part_state* st) {
    return guarded(st, [&](sqc::PartState& p) { return p.set_zero(); });
}

int sqc_part_apply_gates(sqc_part_state* st, const sqc_gate* gates, uint64_t n) {
    return guarded(st, [&](sqc::PartState& p) { return p.apply(gates, n); });
}

int sqc_part_sync(sqc_part_state* st) {
    return guarded(st, [&](sqc::PartState& p) { return p.sync(); });
}

int sqc_part_nnz(sqc_part_state* st, uint64_t* n) {
    if (!n) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::PartState& p) { return p.nnz(n); });
}

int sqc_part_get_state(sqc_part_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n_out,
                       uint32_t flags) {
    return guarded(st, [&](sqc::PartState& p) { return p.get_state(keys, re, im, cap, n_out, flags); });
}

int sqc_part_get_stats(sqc_part_state* st, sqc_part_stats* out) {
    if (!out) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::PartState& p) { return p.stats(out); });
}

const char* sqc_part_last_error(sqc_part_state* st) { return st ? st->p.err.c_str() : ""; }

}  // extern "C"
