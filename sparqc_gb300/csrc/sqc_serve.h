// Serving loop: circuits arrive one at a time and share the GPU with those already running.
//
// A request is planned on submit (as a batch circuit). A step admits queued requests in
// arrival order while a slot is free and their table slice plus gate descriptors fit the
// memory pool, then launches the batch kernel over every resident slot with a deadline: new
// requests start from |0...0>, parked ones resume, and every circuit whose pass ends after the
// deadline parks again. The step waits for the launch and retires the circuits that finished
// (with overlap_steps, the next step does, before it admits and launches). Their states stay
// resident until released.
#pragma once
#include <cstdint>
#include <deque>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/sparqc.h"
#include "sqc_batch.h"
#include "sqc_engine.h"
#include "sqc_pool.h"

namespace sqc {

class Server {
public:
    Server() = default;
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    int init(const sqc_server_options* opt);
    int submit(const sqc_circuit_desc* c, uint64_t* id);
    int step(uint32_t* finished);
    int completed(uint64_t* ids, uint32_t cap, uint32_t* n);
    int request_status(uint64_t id, int* state, int* status);
    int nnz(uint64_t id, uint64_t* out);
    int get_state(uint64_t id, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags);
    int release(uint64_t id);
    int stats(sqc_server_stats* out);
    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    // Table, device control block, live-bucket count, key frame, qubits and precision of a
    // completed request (for comparisons against another state).
    int table_of(uint64_t id, TableDev* t, const Ctl** ctl, unsigned long long* hint, unsigned long long* frame,
                 uint32_t* nq, bool* dbl);
    // The engine of a completed request that ran alone (large circuits), else nullptr.
    Engine* solo_engine(uint64_t id);

    std::string err;

private:
    struct Request {
        CircuitPlan plan;
        int state = SQC_REQ_QUEUED;
        int status = SQC_OK;
        int slot = -1;
        size_t off = 0, bytes = 0;   // pool block (slice, then descriptors and passes)
        unsigned long long nb = 0;
        TableDev table{};
        Ctl ctl{};                   // control block copied back when the request completed
        // a large circuit runs alone on a single-state engine, a slice of its gates per step
        bool solo = false;
        std::unique_ptr<Engine> eng;
        std::vector<sqc_gate> gates;
        uint64_t pos = 0;            // gates applied so far
        uint64_t chunk = 0;          // gates applied in the running step
        double ms_per_gate = 0.0;    // measured on the previous steps
        uint64_t amp_updates = 0;
    };

    int fail(int code, const std::string& msg);
    int cuda(cudaError_t e, const char* what);
    size_t request_bytes(const Request& r) const;
    int admit();
    int admit_solo(uint64_t rid, Request& r);
    size_t solo_bytes(const Request& r) const;
    BatchArgs args(uint32_t n) const;

    int device_ = 0;
    int sms_ = 1;
    bool dbl_ = true;
    PruneBits prune_{};
    double lf_ = 0.45;
    uint32_t min_chunk_ = 8;
    uint32_t max_slots_ = 1024;
    double slice_ms_ = 2.0;
    unsigned long long solo_min_groups_ = 1ULL << 17;
    size_t solo_cap_ = 0, solo_used_ = 0;   // solo_used_ includes the spare engines' tables
    // engines of released large circuits, kept (tables allocated, stream events made) for the
    // next large circuit of the same qubit count and table size; dropped when the memory is needed
    struct Spare {
        std::unique_ptr<Engine> eng;
        uint32_t nq = 0;
        unsigned long long nb = 0;
        size_t bytes = 0;
    };
    std::vector<Spare> spare_;
    static constexpr size_t kMaxSpare = 16;
    uint32_t inject_fail_ = 0;   // admissions left to fail on purpose (sqc_server_options.inject_alloc_failures)
    bool sched_ = false;         // circuits run in schedule_gates order
    // overlap_steps: a step leaves its slice in flight (in_flight_) and retires it at the next
    // call; in_any_ and in_n_ describe the slice's batch launch
    bool overlap_ = false, in_flight_ = false, in_any_ = false;
    uint32_t in_n_ = 0;
    int retire(uint32_t* finished);
    std::vector<uint64_t> solo_;         // running solo requests, in admission order
    double prune_thr_ = 1e-14;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;

    unsigned char* pool_ = nullptr;
    RangePool alloc_;
    BCirc* d_circ_ = nullptr;
    Ctl* d_ctl_ = nullptr;
    BSched* d_sched_ = nullptr;
    unsigned long long* d_words_ = nullptr;
    unsigned* d_cmd_ = nullptr;
    unsigned* d_limit_ = nullptr;
    BatchCtl* d_bctl_ = nullptr;
    BCirc* h_circ_ = nullptr;     // pinned mirrors
    BCirc* stg_circ_ = nullptr;   // what a launch copies to the device, taken from the mirrors at
    unsigned* stg_cmd_ = nullptr; // launch time so that the host may change them while it runs
    unsigned* stg_limit_ = nullptr;
    Ctl* h_ctl_ = nullptr;
    BSched* h_sched_ = nullptr;
    unsigned* h_cmd_ = nullptr;
    unsigned* h_limit_ = nullptr;
    BatchCtl* h_bctl_ = nullptr;

    std::vector<uint64_t> slot_req_;     // request id per slot, 0 = free
    std::vector<uint64_t> in_rid_;       // running request per slot when the slice in flight launched
    std::vector<int> free_slots_;
    uint32_t n_used_ = 0;                // slots [0, n_used_) are scanned by the kernel
    std::deque<uint64_t> queue_;
    std::deque<uint64_t> done_;          // completed, unreleased, in completion order
    std::unordered_map<uint64_t, Request> reqs_;
    uint64_t next_id_ = 1;

    unsigned long long* d_rk_ = nullptr;
    double* d_rr_ = nullptr;
    double* d_ri_ = nullptr;
    size_t rcap_ = 0;

    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, ev2_ = nullptr;
    std::vector<cudaEvent_t> solo_ev_;   // end of each large circuit's part of a step
    uint64_t steps_ = 0, launches_ = 0, upd_done_ = 0;
    double busy_ms_ = 0.0;
};

}  // namespace sqc
