// Host side of the many-circuit batch (kernels in sqc_batch.cu, layout in sqc_batch_types.h).
//
// prepare() plans every circuit on the host (gate resolution and pass split as for a single
// state), bounds the number of 16-key groups each circuit can ever hold from the planner's
// known bits, and gives each circuit a table slice of bound / load_factor buckets (a power of
// two) in one pooled allocation. Because the bound is exact, a slice never has to grow and
// the whole batch runs in one persistent launch without host involvement. run() launches it
// (optionally through a captured CUDA graph); results are read per circuit.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/sparqc.h"
#include "sqc_batch_types.h"
#include "sqc_plan.h"

namespace sqc {

// Blocks per SM that fit for the kernel variant chosen by blocks_per_sm (0: as many as fit).
int batch_residency(bool dbl, int blocks_per_sm);
// The begin kernel and the persistent kernel on `grid` blocks.
cudaError_t launch_batch(const BatchArgs& a, bool dbl, int grid, int blocks_per_sm, unsigned long long deadline_ns,
                         cudaStream_t st);

// Bytes of a table slice of nb buckets (header, keys, amplitudes, list; 256-byte aligned parts).
size_t slice_bytes(unsigned long long nb, bool dbl);
// The table of a slice of nb buckets starting at base (256-byte aligned).
TableDev slice_table(unsigned char* base, unsigned long long nb, bool dbl);
// Buckets of a slice for a circuit that can hold `bound` groups at load factor lf, or 0 when
// more than 2^31 buckets would be needed.
unsigned long long slice_buckets(unsigned long long bound, double lf);

// Plan of one circuit (host).
struct CircuitPlan {
    uint32_t nq = 0;
    std::vector<GateDesc> desc;
    std::vector<BPass> passes;
    Planner end;                   // planner state after the last gate
    unsigned long long bound = 1;  // groups the circuit can ever hold
    uint64_t n_gates = 0;
};

// Plan a circuit from |0...0>. Returns nullptr or the reason it cannot be batched.
const char* plan_circuit(uint32_t nq, const sqc_gate* gates, uint64_t n, uint32_t max_run, uint32_t max_nx,
                         CircuitPlan* out);

class Batch {
public:
    Batch() = default;
    ~Batch();
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;

    int init(const sqc_batch_options* opt);
    int prepare(const sqc_circuit_desc* cs, uint32_t n);
    int run();
    int sync();
    int circuit_status(uint32_t i, int* status);
    int nnz(uint32_t i, uint64_t* out);
    int get_state(uint32_t i, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags);
    // Every circuit's state in one call: circuit i's entries follow circuit i-1's in the
    // arrays, counts[i] of them; one readout kernel per circuit, one copy back per array.
    int get_states(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* counts, uint64_t* total,
                   uint32_t flags);
    int autotune(sqc_batch_tuning* out);
    int stats(sqc_batch_stats* out);
    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    // Table, device control block, live-bucket count, key frame, qubits and precision of
    // circuit i after a synced run (for comparisons against another state).
    int table_of(uint32_t i, TableDev* t, const Ctl** ctl, unsigned long long* hint, unsigned long long* frame,
                 uint32_t* nq, bool* dbl);

    std::string err;

private:
    int fail(int code, const std::string& msg);
    int cuda(cudaError_t e, const char* what);
    int layout();                   // slices for the current plans and tuning
    int plan_and_upload();          // plans of the stored circuits (max_nx_), uploaded, laid out
    int read_ctl();
    int ensure_readout(size_t n);
    void drop_graph();
    BatchArgs args() const;
    int grid() const;

    int device_ = 0;
    int sms_ = 1;
    bool dbl_ = true;
    PruneBits prune_{};
    double lf_ = 0.45;
    uint32_t min_chunk_ = 8;
    unsigned long long idle_limit_ns_ = 2000000000ULL;   // a warp without work for this long ends the run
    uint32_t blocks_per_sm_ = 0;   // 0: occupancy
    bool use_graph_ = false;
    size_t budget_ = 0;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;

    std::vector<CircuitPlan> plans_;
    std::vector<uint32_t> nqs_;                  // the prepared circuits, kept for re-planning
    std::vector<std::vector<sqc_gate>> gates_;   // as applied (schedule_gates order when sched_)
    bool sched_ = false;
    uint32_t max_nx_ = 2;                        // qubits >= 4 a pass may pair across: 1 (pair units) or 2 (quads)
    std::vector<unsigned long long> nb_;

    unsigned char* pool_ = nullptr;
    size_t pool_cap_ = 0, pool_used_ = 0;
    GateDesc* d_desc_ = nullptr;
    size_t desc_cap_ = 0;
    BPass* d_pass_ = nullptr;
    size_t pass_cap_ = 0;
    BCirc* d_circ_ = nullptr;
    Ctl* d_ctl_ = nullptr;
    BSched* d_sched_ = nullptr;
    unsigned long long* d_words_ = nullptr;
    unsigned* d_cmd_ = nullptr;
    unsigned* d_limit_ = nullptr;
    size_t circ_cap_ = 0;
    BatchCtl* d_bctl_ = nullptr;
    Ctl* h_ctl_ = nullptr;          // pinned copy of the control blocks after sync
    BatchCtl* h_bctl_ = nullptr;
    std::vector<TableDev> tables_;

    unsigned long long* d_rk_ = nullptr;
    double* d_rr_ = nullptr;
    double* d_ri_ = nullptr;
    size_t rcap_ = 0;

    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    bool ran_ = false, synced_ = false;
    double last_ms_ = 0.0;
    uint64_t launches_ = 0, runs_ = 0;
    uint64_t epoch_runs_ = 0;   // runs since the slices' headers were last cleared
    static constexpr uint64_t kBatchEpochRestart = 0xFFFFFF00ULL;
};

}  // namespace sqc
