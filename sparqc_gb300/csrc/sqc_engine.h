// Host engine of one sparse state on one GPU: owns the table, the device control block, the
// gate-descriptor buffer and the pass planner. Replaces the reference's TableManager__
// (emulator/device/table_manager.cuh:45-353) and MappingFC__ launchers
// (emulator/device/mapping_GHT.cuh:54-73).
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/sparqc.h"
#include "sqc_measure.h"
#include "sqc_plan.h"
#include "sqc_types.h"

namespace sqc {

struct HostTable {
    Header* hdr = nullptr;
    unsigned long long* keys = nullptr;
    void* amps = nullptr;
    unsigned int* list = nullptr;
    Unit* units = nullptr;
    unsigned long long nb = 0;
};

struct PassRec {
    size_t log_begin;   // replay of this pass starts at this log index...
    Planner snap;       // ...with this planner state
};

class Engine {
public:
    Engine() = default;
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    int init(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt);
    int set_zero();
    // What a caller already knows about the keys it loads: their AND, their OR and their
    // group count (changes of key >> 4 along the array). With it set_state skips its scans.
    struct KeySummary {
        unsigned long long all_and, all_or, groups;
    };
    int set_state(const uint64_t* keys, const double* re, const double* im, uint64_t n,
                  const KeySummary* known = nullptr);
    int apply(const sqc_gate* gates, uint64_t n);
    // hold_last: when the queued gates make more than one pass, the last pass is not launched;
    // its gates stay queued (the planner returns to the state before them), so a caller that
    // feeds a circuit in slices keeps the passes it would get from the whole circuit.
    int flush(bool hold_last = false);
    int sync();
    int nnz(uint64_t* out);
    int get_state(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags);
    // Readout into page-locked host arrays that completes while later work on the state runs:
    // the entries are gathered into the device readout buffers on the state's stream, then
    // copies on a copy stream move them and the count to the host (sqc_get_state_async).
    int get_state_async(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n);
    // Wait for the asynchronous readout in flight (if any); SQC_ERR_CAPACITY if it held more
    // entries than its arrays.
    int readout_wait();
    // Readout of the keys with (key & mask) == value (actual keys, not the stored frame).
    int get_state_where(uint64_t mask, uint64_t value, uint64_t* keys, double* re, double* im, uint64_t cap,
                        uint64_t* n, uint32_t flags);
    int probability(uint64_t mask, uint64_t value, double* p);
    int measure(uint32_t qubit, double u, int* outcome, double* p1);
    int sample(uint64_t shots, uint64_t seed, uint64_t* keys);
    int save(const char* path);
    int load(const char* path);
    int norm2(double* out);
    int compare(Engine& b, double* fidelity, double* max_abs_err);
    // Compare this state (a) with a table that another object owns (b, on the same device,
    // not being modified), of nb_hint live buckets, precision dbl_b and key frame frame_b.
    int compare_with(const TableDev& tb, const Ctl* cb, unsigned long long hint_b, bool dbl_b,
                     unsigned long long frame_b, uint32_t nq_b, int device_b, double* fidelity, double* max_abs_err);
    int stats(sqc_stats* out);
    // Lower the cap on table memory below the HBM budget (bytes; 0 keeps the budget).
    void limit_table_bytes(size_t bytes) {
        if (bytes && bytes < budget_) budget_ = bytes;
    }
    size_t table_budget() const { return budget_; }
    size_t bucket_bytes_now() const { return bucket_bytes(); }
    // After sync() failed with SQC_ERR_BUDGET because the table could not grow: clear the
    // refusal and hand back the gates that did not run. The state is then the output of the
    // last pass that ran, readable and usable as usual.
    int take_unapplied(std::vector<sqc_gate>* rest);
    cudaStream_t stream() const { return stream_; }
    uint32_t nq() const { return nq_; }
    int device() const { return device_; }

    std::string err;

private:
    int fail(int code, const std::string& msg);
    int cuda(cudaError_t e, const char* what);
    int launch_failed(const char* what);
    size_t bucket_bytes() const;
    int alloc_table(unsigned long long nb, HostTable* out);
    void free_table(HostTable* t);
    TableDev dev() const;
    int rebuild(unsigned long long nb_new);
    int repair(size_t failed_pass);
    int ensure_desc(size_t n);
    int ensure_readout(size_t n);
    int readout_buffers_free();   // later users of the readout buffers wait for the async copy
    int ensure_sort(size_t n);
    // wait = false: only queue the readout (the count stays on the device)
    int readout_to_device(uint64_t mask, uint64_t value, bool drop_negl, unsigned long long* got, bool wait = true);
    bool plan_gate(const sqc_gate& g, GateDesc* out);
    int read_ctl();
    int read_sums();   // copy the exact sums back and wait
    int record_event(cudaEvent_t* out);
    void harvest_events();
    unsigned long long max_groups() const;

    int device_ = 0;
    int sms_ = 1;
    uint32_t nq_ = 0;
    bool dbl_ = true;
    double thr_ = 1e-14;
    bool dev_upd_only_ = false;     // amp updates count device-applied gates only
    bool sched_ = false;            // each apply() call's gates go in schedule_gates order
    // asynchronous readout: copy stream, gathered / copied events, count word
    cudaStream_t copy_stream_ = nullptr;
    cudaEvent_t ev_gathered_ = nullptr, ev_copied_ = nullptr;
    unsigned long long* h_async_n_ = nullptr;   // page-locked: the gathered count, once copied
    uint64_t async_cap_ = 0, async_expect_ = 0;
    bool async_pending_ = false;
    unsigned long long epochs_ = 0; // epochs since the table's headers were last cleared
    int next_epoch();
    std::vector<uint32_t> perm_;    // its scratch
    double lf_ = 0.5;
    uint32_t max_run_ = kMaxRun;
    uint32_t max_nx_ = 2;        // cross-group qubits per pass at most
    size_t budget_ = 0;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;

    HostTable tab_;
    Ctl* ctl_ = nullptr;        // device
    Ctl* ctl_host_ = nullptr;   // pinned mirror
    ExactSums* sums_ = nullptr;       // device: exact sums of norm, probability and compare
    ExactSums* sums_host_ = nullptr;  // pinned mirror
    unsigned long long seq_verified_ = 0;
    unsigned long long list_hint_ = 1;
    PruneBits prune_{};

    Planner plan_;              // after every queued gate
    Planner snap_plan_;         // right after the last launched device gate...
    size_t snap_log_ = 0;       // ...whose source gate precedes this log index
    unsigned long long host_upd_ = 0;   // amp updates credited on the host (resolved trailing gates)

    std::vector<sqc_gate> pending_;   // queued, not launched
    std::vector<sqc_gate> log_;       // launched since the last verified sync
    std::vector<PassRec> passes_;     // passes launched since the last verified sync

    GateDesc* d_desc_ = nullptr;
    GateDesc* h_desc_ = nullptr;
    TinyPass* d_tiny_ = nullptr;    // pass records of single-launch flushes (tiny states)
    TinyPass* h_tiny_ = nullptr;
    size_t desc_cap_ = 0, desc_used_ = 0;

    unsigned long long* d_rk_ = nullptr;
    double* d_rr_ = nullptr;
    double* d_ri_ = nullptr;
    size_t rcap_ = 0;
    SortBuffers sort_;            // device key sort of readouts (sorted readout, sampling)
    size_t sort_cap_ = 0;

    uint64_t gates_applied_ = 0, passes_run_ = 0, launches_ = 0, replays_ = 0, rebuilds_ = 0;
    uint64_t passes_pair_ = 0;

    // pass timing (time_passes): an event before the first pass of a flush and one after every
    // pass; each timed pass spans [before, after], the after event of the pass before it being
    // its before event
    struct TimedPass {
        cudaEvent_t before, after;
        bool pair;
    };
    bool time_passes_ = false;
    std::vector<cudaEvent_t> ev_free_, ev_all_;
    std::vector<TimedPass> timed_;
    uint64_t pass_ns_pair_ = 0, pass_ns_stream_ = 0;
};

}  // namespace sqc
