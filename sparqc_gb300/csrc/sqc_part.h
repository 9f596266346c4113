// A state allowed to outgrow the device: the reference's "PC" mode (part of the circuit on one
// GPU, circuit size > GPU memory; emulator/device/device_data.cuh:20-23), which the reference
// describes but never built (its subtable code, emulator/device/device_table_PCS.cuh:26-583,
// is commented out).
//
// The state lives in one device table while it fits. When a pass cannot grow the table within
// the device budget, the state that the passes before it produced moves to host memory and the
// remaining gates run in windows over partitions:
//  * a window is a run of gates whose non-diagonal gates (X, Y, H, Rx, Ry, U) target no qubit
//    of a set P of partition qubits; P holds qubits >= 4 whose values vary across the keys;
//  * no gate of the window changes a key's P bits, so the state splits into 2^|P| partitions by
//    those bits and every partition runs through the device table alone: loaded, all the
//    window's gates applied (controls and diagonal gates on P qubits act per key as usual),
//    read back. Per-key results are the same as in one table: every update reads one key or a
//    pair that differs in a non-P bit, and pruning is per key;
//  * a partition that outgrows the device during its window is read back at the pass that could
//    not grow and split by one more qubit (again >= 4, varying, and untouched by the window's
//    non-diagonal gates); the halves continue with the gates that had not run.
// Qubits >= 4 keep a 16-key group inside one partition, so a partition's group count is exact
// and its table is sized from it. When the whole state fits comfortably again, it returns to
// the device. Host-side state lives in page-locked buffers (copies run at the link's speed),
// recycled through a pool; the split of the state into partitions runs on all host cores.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sparqc.h"
#include "sqc_engine.h"

namespace sqc {

// Page-locked host blocks, kept for reuse once released (pinning is paid once). Falls back to
// pageable memory when the system refuses to pin more.
class PinnedPool {
public:
    PinnedPool() = default;
    PinnedPool(const PinnedPool&) = delete;
    PinnedPool& operator=(const PinnedPool&) = delete;
    ~PinnedPool();
    void* get(size_t bytes);   // nullptr when no memory is left
    void put(void* p);

private:
    struct Block {
        size_t bytes;
        bool pinned;
    };
    std::multimap<size_t, void*> free_;
    std::unordered_map<void*, Block> blocks_;
};

// Keys (each 16-key group contiguous, as readouts emit them) and their amplitudes, in one
// pooled block: keys, then re, then im.
struct Run {
    uint64_t* k = nullptr;
    double* r = nullptr;
    double* i = nullptr;
    uint64_t n = 0;
    uint64_t groups = 0;
    uint64_t all_and = ~0ULL, all_or = 0;

    Run() = default;
    Run(const Run&) = delete;
    Run& operator=(const Run&) = delete;
    Run(Run&& o) noexcept { take(o); }
    Run& operator=(Run&& o) noexcept {
        if (this != &o) {
            release();
            take(o);
        }
        return *this;
    }
    ~Run() { release(); }
    bool alloc(PinnedPool* pool, uint64_t count);
    void release();
    // AND, OR and group count of the keys, on `threads` host threads
    void fill_summary(int threads);

private:
    void take(Run& o);
    PinnedPool* pool_ = nullptr;
    void* block_ = nullptr;
};

class PartState {
public:
    int init(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt, uint64_t device_bytes);
    int set_zero();
    int apply(const sqc_gate* gates, uint64_t n);
    int sync();
    int nnz(uint64_t* out);
    int get_state(uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n, uint32_t flags);
    int stats(sqc_part_stats* out);

    std::string err;

private:
    int fail(int code, const std::string& msg);
    int from_engine(int rc);
    int read_engine(Run* out);
    int load_engine(const Run& in);
    int run_windows();
    int run_bin(Run& in, std::vector<sqc_gate> gates, unsigned long long free_bits, std::vector<Run>* out);
    int distribute(std::vector<Run>& runs, const std::vector<int>& bits, std::vector<Run>* bins);
    uint64_t bin_keys_target() const;
    void take_counters();
    int maybe_return();

    PinnedPool pool_;   // destroyed after the runs that hold its blocks
    Engine eng_;
    uint32_t nq_ = 0;
    double thr_ = 1e-14;
    int threads_ = 1;
    bool resident_ = true;
    std::vector<Run> runs_;
    std::vector<sqc_gate> pending_;
    uint32_t last_bits_ = 0;
    uint64_t spills_ = 0, windows_ = 0, bins_ = 0, splits_ = 0, returns_ = 0;
    uint64_t h2d_ = 0, d2h_ = 0, upd_ = 0, max_bin_ = 0;
};

}  // namespace sqc
