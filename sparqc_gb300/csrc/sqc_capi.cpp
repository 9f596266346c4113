// extern "C" entry points of include/sparqc.h. Every call returns a status code; no C++
// exception crosses the boundary (the reference throws std::string on the host and exits on
// CUDA errors, emulator/device/table_manager.cuh:175-259, emulator/third_party/helper_cuda.h).
#include <new>
#include <string>
#include <vector>

#include "../../include/sparqc.h"
#include "sqc_handles.h"
#include "sqc_kernels.h"
#include "sqc_plan.h"
#include "sqc_twoq.h"

namespace {

template <class F>
int guarded(sqc_state* st, F&& f) {
    if (!st) return SQC_ERR_ARG;
    try {
        return f(st->eng);
    } catch (const std::bad_alloc&) {
        st->eng.err = "host allocation failed";
        return SQC_ERR_OOM;
    } catch (...) {
        st->eng.err = "unexpected host exception";
        return SQC_ERR_STATE;
    }
}

int one(sqc_state* st, uint32_t kind, uint32_t t, double par) {
    sqc_gate g;
    g.kind = kind;
    g.target = t;
    g.controls = 0;
    g.theta = par;
    g.phi = 0.0;
    g.lambda = 0.0;
    return guarded(st, [&](sqc::Engine& e) { return e.apply(&g, 1); });
}

}  // namespace

extern "C" {

void sqc_default_options(sqc_options* opt) {
    if (!opt) return;
    opt->precision = SQC_FP64;
    opt->prune_threshold = 1e-14;
    opt->load_factor = 0.5;
    opt->initial_buckets = 0;
    opt->stream = nullptr;
    opt->device = 0;
    opt->max_fused_gates = 0;
    opt->time_passes = 0;
    opt->max_cross_qubits = 0;
    opt->device_updates_only = 0;
    opt->schedule_gates = 0;
}

int sqc_create(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt, sqc_state** out) {
    if (!out) return SQC_ERR_ARG;
    *out = nullptr;
    sqc_state* st = nullptr;
    try {
        st = new sqc_state();
    } catch (...) {
        return SQC_ERR_OOM;
    }
    int rc;
    try {
        rc = st->eng.init(nq, params, opt);
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

int sqc_destroy(sqc_state* st) {
    delete st;
    return SQC_OK;
}

int sqc_set_zero_state(sqc_state* st) { return guarded(st, [](sqc::Engine& e) { return e.set_zero(); }); }

int sqc_set_state(sqc_state* st, const uint64_t* keys, const double* re, const double* im, uint64_t n) {
    return guarded(st, [&](sqc::Engine& e) { return e.set_state(keys, re, im, n); });
}

int sqc_apply_gates(sqc_state* st, const sqc_gate* gates, uint64_t n) {
    return guarded(st, [&](sqc::Engine& e) { return e.apply(gates, n); });
}

int sqc_x(sqc_state* st, uint32_t t) { return one(st, SQC_X, t, 0.0); }
int sqc_y(sqc_state* st, uint32_t t) { return one(st, SQC_Y, t, 0.0); }
int sqc_z(sqc_state* st, uint32_t t) { return one(st, SQC_Z, t, 0.0); }
int sqc_h(sqc_state* st, uint32_t t) { return one(st, SQC_H, t, 0.0); }
int sqc_phase(sqc_state* st, uint32_t t, double par) { return one(st, SQC_PHASE, t, par); }
int sqc_rz(sqc_state* st, uint32_t t, double par) { return one(st, SQC_RZ, t, par); }
int sqc_rx(sqc_state* st, uint32_t t, double par) { return one(st, SQC_RX, t, par); }
int sqc_ry(sqc_state* st, uint32_t t, double par) { return one(st, SQC_RY, t, par); }

int sqc_flush(sqc_state* st) { return guarded(st, [](sqc::Engine& e) { return e.flush(); }); }

int sqc_sync(sqc_state* st) { return guarded(st, [](sqc::Engine& e) { return e.sync(); }); }

int sqc_nnz(sqc_state* st, uint64_t* nnz) {
    if (!nnz) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) { return e.nnz(nnz); });
}

int sqc_get_state(sqc_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags) {
    return guarded(st, [&](sqc::Engine& e) { return e.get_state(keys, re, im, cap, n, flags); });
}

int sqc_get_state_async(sqc_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n) {
    return guarded(st, [&](sqc::Engine& e) { return e.get_state_async(keys, re, im, cap, n); });
}

int sqc_readout_wait(sqc_state* st) {
    return guarded(st, [&](sqc::Engine& e) { return e.readout_wait(); });
}

int sqc_norm2(sqc_state* st, double* norm2) {
    if (!norm2) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) { return e.norm2(norm2); });
}

int sqc_compare(sqc_state* a, sqc_state* b, double* fidelity, double* max_abs_err) {
    if (!b || !fidelity || !max_abs_err) return SQC_ERR_ARG;
    return guarded(a, [&](sqc::Engine& e) { return e.compare(b->eng, fidelity, max_abs_err); });
}

int sqc_swap(sqc_state* st, uint32_t a, uint32_t b) {
    if (a == b) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) -> int {
        sqc_gate g[3];
        const uint32_t tgt[3] = {b, a, b}, ctl[3] = {a, b, a};
        for (int i = 0; i < 3; ++i) {
            g[i].kind = SQC_X;
            g[i].target = tgt[i];
            g[i].controls = 1ULL << (ctl[i] & 63);
            g[i].theta = g[i].phi = g[i].lambda = 0.0;
        }
        if (a >= e.nq() || b >= e.nq()) return (int)SQC_ERR_ARG;
        return e.apply(g, 3);
    });
}

int sqc_save(sqc_state* st, const char* path) {
    if (!path) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) { return e.save(path); });
}

int sqc_load(sqc_state* st, const char* path) {
    if (!path) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) { return e.load(path); });
}

int sqc_get_state_where(sqc_state* st, uint64_t mask, uint64_t value, uint64_t* keys, double* re, double* im,
                        uint64_t cap, uint64_t* n, uint32_t flags) {
    return guarded(st, [&](sqc::Engine& e) { return e.get_state_where(mask, value, keys, re, im, cap, n, flags); });
}

int sqc_probability(sqc_state* st, uint64_t mask, uint64_t value, double* p) {
    return guarded(st, [&](sqc::Engine& e) { return e.probability(mask, value, p); });
}

int sqc_measure(sqc_state* st, uint32_t qubit, double u, int* outcome, double* p1) {
    return guarded(st, [&](sqc::Engine& e) { return e.measure(qubit, u, outcome, p1); });
}

int sqc_sample(sqc_state* st, uint64_t shots, uint64_t seed, uint64_t* keys) {
    return guarded(st, [&](sqc::Engine& e) { return e.sample(shots, seed, keys); });
}

int sqc_get_stats(sqc_state* st, sqc_stats* out) {
    if (!out) return SQC_ERR_ARG;
    return guarded(st, [&](sqc::Engine& e) { return e.stats(out); });
}

int sqc_twoq_gates(uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta, double phi,
                   const double* u, sqc_gate* out, uint64_t cap, uint64_t* n) {
    if (!n) return SQC_ERR_ARG;
    *n = 0;
    std::vector<sqc_gate> g;
    const int rc = sqc::twoq_sequence(form, a, b, c, controls, theta, phi, u, g);
    if (rc) return rc;
    *n = g.size();
    if (g.size() > cap) return SQC_ERR_CAPACITY;
    if (!g.empty() && !out) return SQC_ERR_ARG;
    for (size_t i = 0; i < g.size(); ++i) out[i] = g[i];
    return SQC_OK;
}

int sqc_schedule_gates(uint32_t nq, const sqc_gate* gates, uint64_t n, uint32_t max_cross_qubits, uint32_t* perm) {
    if (nq < 1 || nq > 64 || max_cross_qubits < 1 || max_cross_qubits > 3 || (n && (!gates || !perm)) ||
        n > sqc::kScheduleMaxGates)
        return SQC_ERR_ARG;
    for (uint64_t i = 0; i < n; ++i)
        if (sqc::check_gate(gates[i], nq)) return SQC_ERR_ARG;
    sqc::schedule_gates(gates, (size_t)n, max_cross_qubits, sqc::kMaxRun, sqc::kScheduleWindow, perm);
    return SQC_OK;
}

int sqc_apply_twoq(sqc_state* st, uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta,
                   double phi, const double* u) {
    return guarded(st, [&](sqc::Engine& e) {
        std::vector<sqc_gate> g;
        const int rc = sqc::twoq_sequence(form, a, b, c, controls, theta, phi, u, g);
        if (rc) {
            e.err = "bad two-qubit gate (qubits, controls, form or matrix)";
            return rc;
        }
        return e.apply(g.data(), g.size());
    });
}

int sqc_fp64_rate(uint32_t device, double* fma_per_s) {
    if (!fma_per_s) return SQC_ERR_ARG;
    *fma_per_s = 0.0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || (int)device >= ndev) return SQC_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice((int)device) != cudaSuccess) return SQC_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, (int)device);
    const cudaError_t e = sqc::measure_fp64_rate(sms, fma_per_s);
    cudaSetDevice(prev);
    return e == cudaSuccess ? SQC_OK : SQC_ERR_CUDA;
}

const char* sqc_status_string(int status) {
    switch (status) {
    case SQC_OK: return "ok";
    case SQC_ERR_ARG: return "bad argument";
    case SQC_ERR_OOM: return "out of memory";
    case SQC_ERR_TABLE_FULL: return "table full";
    case SQC_ERR_CUDA: return "CUDA error";
    case SQC_ERR_BUDGET: return "HBM budget exceeded";
    case SQC_ERR_CAPACITY: return "output capacity too small";
    case SQC_ERR_NO_DEVICE: return "no suitable CUDA device";
    case SQC_ERR_STATE: return "handle in an unusable state";
    default: return "unknown status";
    }
}

const char* sqc_last_error(sqc_state* st) { return st ? st->eng.err.c_str() : "null handle"; }

void* sqc_stream(sqc_state* st) { return st ? (void*)st->eng.stream() : nullptr; }

}  // extern "C"
