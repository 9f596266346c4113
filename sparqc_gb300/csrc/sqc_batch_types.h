// Data shared by the host and the kernels of the many-circuit batch (no device code).
//
// A batch holds up to a few thousand independent circuits, each with its own table slice
// (the single-state layout of sqc_device.cuh, sized from the circuit's group bound), its own
// control block (Ctl) and gate descriptors. One persistent kernel runs every circuit's
// passes: a circuit's pass is cut into chunks of list entries; any warp may take any chunk
// of any circuit, and the warp that finishes the last chunk of a pass publishes it and opens
// the circuit's next pass. Circuits never wait for one another.
#pragma once
#include <cstdint>

#include "sqc_types.h"

namespace sqc {

// One pass of a circuit: gates [g0, g1) of its descriptors.
struct BPass {
    uint32_t g0, g1;
    uint16_t nx;          // cross-group qubits: 0, 1 or 2
    uint16_t keys_fixed;  // diagonal gates only
    uint8_t q1, q2;       // the cross-group qubits (>= 4; unused ones 0xFF)
    uint8_t pad[2];
};

// A circuit of the batch (read-only while the kernel runs).
struct BCirc {
    TableDev t;                    // its table slice (units unused)
    const GateDesc* gates;
    const BPass* passes;
    uint32_t npasses;
    uint32_t pad;
    unsigned long long max_groups;  // groups the slice takes (0.9 of its buckets)
    unsigned long long bound;       // groups the circuit can ever hold (host-side bound)
};

// Scheduling word of a circuit: (pass << 44) | (chunks << 22) | chunks issued. A warp takes a
// chunk with one atomicAdd; the chunk is valid iff issued < chunks in the returned word.
constexpr int kSchedFieldBits = 22;
constexpr unsigned long long kSchedFieldMask = (1ULL << kSchedFieldBits) - 1;
constexpr unsigned long long kMaxChunks = (1ULL << (kSchedFieldBits - 1)) - 1;   // room for over-issue
constexpr uint32_t kMaxBatchPasses = (1u << 20) - 1;

enum BState : unsigned int { BS_IDLE = 0, BS_RUN = 1, BS_DONE = 2, BS_PARKED = 3, BS_FAILED = 4 };

struct alignas(32) BSched {
    unsigned int done;         // chunks finished in the current pass
    unsigned int chunk;        // list entries per chunk in the current pass (a multiple of 4)
    unsigned int next_total;   // chunks of the pass a parked circuit resumes with
    unsigned int state;        // BState
    unsigned int limit;        // the circuit parks before starting this pass
    unsigned int pad[3];
};

// Batch control block.
struct BatchCtl {
    unsigned int status;            // ST_TIMEOUT when a warp found no work for too long
    unsigned int left;              // circuits still running in this launch
    unsigned int epoch;             // table epoch of the last reset
    unsigned int pad;
    unsigned long long deadline_ns; // %globaltimer after which circuits park at their next pass (0: none)
    unsigned long long progress;    // passes published
};

// Per-circuit command of the begin kernel.
enum BCmd : unsigned int { BC_KEEP = 0, BC_INIT = 1, BC_RESUME = 2 };

struct BatchArgs {
    const BCirc* circ;
    Ctl* ctl;
    BSched* sched;
    unsigned long long* words;      // scheduling word per circuit (dense: warps scan them)
    BatchCtl* bctl;
    const unsigned int* cmd;        // begin kernel: BCmd per circuit
    const unsigned int* limit;      // begin kernel: pass limit per circuit
    uint32_t n;                     // circuits
    uint32_t amp_bytes;             // 16 (FP64) or 8 (FP32)
    uint32_t min_chunk;             // list entries per chunk at least (a multiple of 4)
    uint32_t target_chunks;         // chunks per pass at most, for large circuits
    PruneBits prune;
    unsigned long long idle_limit_ns;   // a warp that finds no work for this long records ST_TIMEOUT
};

}  // namespace sqc
