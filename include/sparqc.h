/*
 * sparqc.h -- C ABI of the GB300 sparse statevector gate engine.
 *
 * The state is a GPU open-addressing hash table mapping 64-bit basis-state keys to complex
 * amplitudes. Gates are applied by pairing each key with k ^ (1 << target), updating the
 * pair with its 2x2 matrix, writing the results back into the table and pruning negligible
 * amplitudes after branching gates. All entry points take plain pointers and sizes, return
 * an int status (SQC_OK = 0) and never throw.
 *
 * Reference interface replaced (ivanNovikau/SparQC, header-only C++, no C ABI of its own):
 *   Circuit__(nq, hash_table_parameters)      emulator/include/circuit.h:34-43
 *   x/y/z/h(t), phase/rz/rx/ry(t, par)         emulator/include/circuit.h:45-83
 *   TableManager__::gate_sq / gate_sq_par      emulator/device/table_manager.cuh:311-340
 *   set_zero_quantum_state                     emulator/device/table_manager.cuh:299-308
 *   get_statevector (readout)                  emulator/device/table_manager.cuh:343-350,
 *                                              emulator/device/table.cuh:47-75
 *   hash_table_parameters                      emulator/include/sim_parameters_types.h:133-145
 * The C++ drop-in class with the reference's names is in sparqc_circuit.hpp.
 *
 * Threading: a handle is bound to one CUDA stream and is not thread-safe; separate handles
 * may be used from separate threads. Gate calls are asynchronous and may be buffered so
 * that consecutive gates are fused into one device pass; sqc_sync, readout, nnz and norm
 * queries flush and wait.
 */
#ifndef SPARQC_H
#define SPARQC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
enum {
    SQC_OK = 0,
    SQC_ERR_ARG = 1,        /* bad argument (qubit out of range, target among controls, ...) */
    SQC_ERR_OOM = 2,        /* device allocation failed */
    SQC_ERR_TABLE_FULL = 3, /* probe limit reached and the table could not grow */
    SQC_ERR_CUDA = 4,       /* CUDA runtime error (message in sqc_last_error) */
    SQC_ERR_BUDGET = 5,     /* table memory would exceed the HBM budget */
    SQC_ERR_CAPACITY = 6,   /* caller buffer too small (required size returned) */
    SQC_ERR_NO_DEVICE = 7,  /* no CUDA device, or more devices requested than present */
    SQC_ERR_STATE = 8       /* handle in an unusable state */
};

/* ---- gates --------------------------------------------------------------------------- */
/* Kinds 0-7 are the reference's gates with the reference's argument meaning:
 * phase(t, par) multiplies the bit-1 amplitude by e^{i par}; rz/rx/ry(t, par) rotate by par
 * (cos/sin of par/2 are applied, emulator/device/table_manager.cuh:333-336).
 * Kinds 8-12 are additions: S, Sdg (exact +-i on the bit-1 amplitude), T, Tdg (Phase with
 * cos = +-sin = sqrt(1/2)) and U(theta, phi, lambda), the u3 matrix
 * [[cos(theta/2), -e^{i lambda} sin(theta/2)], [e^{i phi} sin(theta/2), e^{i(phi+lambda)} cos(theta/2)]]. */
enum {
    SQC_X = 0, SQC_Y = 1, SQC_Z = 2, SQC_H = 3,
    SQC_PHASE = 4, SQC_RZ = 5, SQC_RX = 6, SQC_RY = 7,
    SQC_S = 8, SQC_SDG = 9, SQC_T = 10, SQC_TDG = 11, SQC_U = 12
};

typedef struct sqc_gate {
    uint32_t kind;      /* SQC_X ... SQC_U */
    uint32_t target;    /* target qubit: bit `target` of the key, qubit 0 = least significant */
    uint64_t controls;  /* control mask: the gate acts on a key iff (key & controls) == controls */
    double theta;       /* angle for phase/rz/rx/ry/u */
    double phi;         /* u only */
    double lambda;      /* u only */
} sqc_gate;             /* 40 bytes */

/* ---- construction -------------------------------------------------------------------- */
/* Mirrors hash_table_parameters (emulator/include/sim_parameters_types.h:133-145).
 * N_devices must be 1 (one GPU per state). coef_gpu_memory_reserve is the fraction of the
 * device memory left free: tables may use at most (1 - reserve) * total memory.
 * N_subtables and log2_N_bucket_spots are accepted for compatibility and ignored: buckets
 * here always hold 16 keys (128 bytes of keys). */
typedef struct sqc_hash_table_parameters {
    uint32_t N_devices;
    double coef_gpu_memory_reserve;
    uint32_t N_subtables;
    uint32_t log2_N_bucket_spots;
} sqc_hash_table_parameters;

enum { SQC_FP64 = 64, SQC_FP32 = 32 };

typedef struct sqc_options {
    uint32_t precision;        /* SQC_FP64 (default) or SQC_FP32 amplitudes */
    double prune_threshold;    /* > 0, default 1e-14: prune iff |re| < thr && |im| < thr (in FP64) */
    double load_factor;        /* target groups per bucket after growth, default 0.5 */
    uint64_t initial_buckets;  /* initial bucket count (rounded to a power of two), 0 = 1024 */
    void* stream;              /* cudaStream_t to run on; NULL = the handle creates its own */
    uint32_t device;           /* CUDA device ordinal, default 0 */
    uint32_t max_fused_gates;  /* cap on gates fused into one pass, 0 = default (64) */
    uint32_t time_passes;      /* 1: bracket every gate pass with CUDA events on the handle's stream
                                  (sqc_stats.pass_ns_*); the events keep consecutive passes from
                                  overlapping one's launch with the other's drain, and cost ~4-9%
                                  of a many-pass circuit. 0 (default): no events */
    uint32_t max_cross_qubits; /* qubits >= 4 one pass may pair keys across (branching or swap gates on
                                  them), 1, 2 or 3; 0 = default (3 for FP32, 2 for FP64). Results do
                                  not depend on it. */
    uint32_t device_updates_only; /* 1: sqc_stats.amp_updates counts only gates the device applied;
                                  0 (default): gates the host resolved without touching the state
                                  (a known-zero control, an uncontrolled X as a relabelling of the
                                  keys, a one-sided diagonal gate on a known-zero bit) count too,
                                  each with the key count it acted on, as in the reference, which
                                  runs every gate on the device */
    uint32_t schedule_gates;   /* 1: each gate array given to sqc_apply_gates is applied in the order
                                  sqc_schedule_gates gives it (max_cross_qubits as above): gates move
                                  ahead of gates they commute with, so passes fuse more of them. The
                                  state is the same in exact arithmetic; rounding and pruning follow
                                  the new order, so results are no longer bit-identical to the
                                  reference's. 0 (default): the order given */
} sqc_options;

typedef struct sqc_state sqc_state;

/* Fill *opt with the defaults. */
void sqc_default_options(sqc_options* opt);

/* Create a state of nq qubits (1..64) set to |0...0>. params may be NULL (defaults), opt may
 * be NULL (defaults). Replaces Circuit__::Circuit__ + TableManager__ construction. */
int sqc_create(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt,
               sqc_state** out);
int sqc_destroy(sqc_state* st);

/* |0...0>: key 0 with amplitude 1. Replaces TableManager__::set_zero_quantum_state. */
int sqc_set_zero_state(sqc_state* st);

/* Load n distinct (key, re, im) entries from host memory (amplitudes rounded to the state's
 * precision). Keys must fit in nq bits. */
int sqc_set_state(sqc_state* st, const uint64_t* keys, const double* re, const double* im,
                  uint64_t n);

/* ---- gates --------------------------------------------------------------------------- */
/* Queue n gates (host array). Asynchronous. Replaces TableManager__::gate_sq/gate_sq_par. */
int sqc_apply_gates(sqc_state* st, const sqc_gate* gates, uint64_t n);

/* SWAP of qubits a and b (no counterpart in the reference): queued as the three CNOTs
 * CX(a->b) CX(b->a) CX(a->b), each a controlled X, so it is exact. */
int sqc_swap(sqc_state* st, uint32_t a, uint32_t b);

/* One-gate conveniences with the reference's names (emulator/include/circuit.h:45-83),
 * uncontrolled. */
int sqc_x(sqc_state* st, uint32_t t);
int sqc_y(sqc_state* st, uint32_t t);
int sqc_z(sqc_state* st, uint32_t t);
int sqc_h(sqc_state* st, uint32_t t);
int sqc_phase(sqc_state* st, uint32_t t, double par);
int sqc_rz(sqc_state* st, uint32_t t, double par);
int sqc_rx(sqc_state* st, uint32_t t, double par);
int sqc_ry(sqc_state* st, uint32_t t, double par);

/* Launch everything queued without waiting (the work is ordered on the handle's stream). */
int sqc_flush(sqc_state* st);

/* Launch everything queued, wait for it, check the device status word, grow the tables and
 * replay if a pass ran out of table space. */
int sqc_sync(sqc_state* st);

/* ---- readout ------------------------------------------------------------------------- */
enum { SQC_READ_SORTED = 1, SQC_READ_DROP_NEGLIGIBLE = 2 };

/* Number of keys held (present entries, including any kept negligible ones). */
int sqc_nnz(sqc_state* st, uint64_t* nnz);

/* Copy the state into caller arrays of capacity cap. flags: SQC_READ_SORTED orders by key;
 * SQC_READ_DROP_NEGLIGIBLE drops |re|,|im| < threshold entries as the reference's readout
 * does (emulator/device/table.cuh:47-75). *n receives the count; if it exceeds cap the call
 * returns SQC_ERR_CAPACITY and copies nothing. */
int sqc_get_state(sqc_state* st, uint64_t* keys, double* re, double* im, uint64_t cap,
                  uint64_t* n, uint32_t flags);

/* Asynchronous readout (no counterpart in the reference): as sqc_get_state without flags, into
 * page-locked host arrays (cudaHostAlloc, cudaMallocHost or cudaHostRegister; *n too). The
 * state's entries are gathered into a device buffer on the state's stream, and a copy on a
 * stream of the state's own writes them to the host, so work queued on the state afterwards (a
 * new circuit, more gates) runs while they travel. The arrays and *n hold the result once
 * sqc_readout_wait returns, which returns SQC_ERR_CAPACITY if the state held more than cap
 * entries (the first cap are written). The next sqc_get_state_async first completes the
 * previous one as sqc_readout_wait does (returning its error); other readouts and
 * sqc_set_state wait on the device for the copy before reusing the buffer. SQC_ERR_ARG for
 * arrays that are not page-locked. */
int sqc_get_state_async(sqc_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n);
/* Wait for the state's asynchronous readout in flight, if any. */
int sqc_readout_wait(sqc_state* st);

/* Sum of |amplitude|^2, accumulated in FP64 on the device. */
int sqc_norm2(sqc_state* st, double* norm2);

/* ---- snapshots ------------------------------------------------------------------------ */
/* Write the state to a file / replace the state with a file's (no counterpart in the
 * reference, which names _RESTART.hdf5 files, emulator/include/QLib.h:39-40, but never writes
 * them). Plain binary, little endian: the 8 bytes "SQCSNAP1", uint32 nq, uint32 precision,
 * uint64 n, then n uint64 keys sorted ascending, n double re, n double im. Loading needs the
 * same qubit count; amplitudes are rounded to the state's precision. */
int sqc_save(sqc_state* st, const char* path);
int sqc_load(sqc_state* st, const char* path);

/* ---- selection and measurement ---------------------------------------------------------- */
/* Readout restricted to the keys with (key & mask) == value, as sqc_get_state (flags
 * SQC_READ_SORTED sorts by key on the device). The reference's Circuit__::get_state_full
 * selects states by a per-qubit pattern (state_to_choose: -1 any, 0, 1;
 * emulator/include/circuit.h:206-253): its qubits fixed to 0 or 1 are the mask bits, their
 * values the value bits. */
int sqc_get_state_where(sqc_state* st, uint64_t mask, uint64_t value, uint64_t* keys, double* re, double* im,
                        uint64_t cap, uint64_t* n, uint32_t flags);
/* Sum of |amplitude|^2 over the keys with (key & mask) == value (FP64, on the device). */
int sqc_probability(sqc_state* st, uint64_t mask, uint64_t value, double* p);
/* Projective measurement of one qubit (no counterpart in the reference): outcome 1 iff
 * u < p1, p1 = probability of reading 1 divided by the norm; the keys of the other outcome are
 * removed and the remaining amplitudes multiplied by 1/sqrt(their total probability).
 * u must be in [0, 1); *p1 (may be NULL) receives p1. */
int sqc_measure(sqc_state* st, uint32_t qubit, double u, int* outcome, double* p1);
/* shots basis states drawn with probability |amplitude|^2 / norm (no counterpart in the
 * reference): the keys are sorted, their probabilities summed into a cumulative distribution,
 * and shot s takes the first key whose cumulative probability exceeds u_s * total, with u_s a
 * splitmix64 hash of (seed, s). The same state and seed give the same samples. */
int sqc_sample(sqc_state* st, uint64_t shots, uint64_t seed, uint64_t* keys);

/* ---- two-qubit gates ------------------------------------------------------------------ */
/* No counterpart in the reference (its gates are eight uncontrolled single-qubit gates,
 * emulator/include/circuit.h:45-83). A two-qubit gate on qubits (a, b) acts on the basis states
 * indexed i_a + 2 i_b and is applied as a short sequence of this engine's own gates, which fuse
 * into the usual passes:
 *   SQC_2Q_UNITARY  any 4x4 unitary u (row-major (re, im) pairs, unitary to 1e-9): two-level
 *                   rotations (controlled U and Phase gates) and a phase, at most 13 gates that
 *                   act on amplitudes plus relabellings; results agree with the matrix to ~1e-15;
 *   SQC_2Q_RZZ      exp(-i theta/2 Z_a Z_b), two controlled Rz;
 *   SQC_2Q_ISWAP    [[1,0,0,0],[0,0,i,0],[0,i,0,0],[0,0,0,1]], exact (CNOTs and S);
 *   SQC_2Q_FSIM     [[1,0,0,0],[0,cos t,-i sin t,0],[0,-i sin t,cos t,0],[0,0,0,e^{-i phi}]];
 *   SQC_2Q_CSWAP    swap of a and b where qubit c is 1 (Fredkin), exact (three X gates);
 *   SQC_2Q_SWAP     swap of a and b, exact.
 * Every gate applies only where all `controls` bits are 1 (they may not include a, b or c). */
enum { SQC_2Q_UNITARY = 0, SQC_2Q_RZZ = 1, SQC_2Q_ISWAP = 2, SQC_2Q_FSIM = 3, SQC_2Q_CSWAP = 4, SQC_2Q_SWAP = 5 };
/* The gate sequence of one two-qubit gate (c: CSWAP's control qubit, else ignored; u: the
 * matrix of SQC_2Q_UNITARY, else ignored) into out (capacity cap; 32 always suffice); *n
 * receives the count. For batches, servers and partitioned states, which take gate arrays. */
int sqc_twoq_gates(uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta, double phi,
                   const double* u, sqc_gate* out, uint64_t cap, uint64_t* n);
/* An order of a gate array that gate passes fuse better, as a permutation: perm[i] receives the
 * index of the i-th gate to apply. Gates move ahead only of gates they commute with (neither
 * changes a qubit the other touches: a gate changes its target unless it is diagonal, and only
 * reads its controls), so the state is the same in exact arithmetic; rounding and pruning follow
 * the new order. Passes are built greedily from the first gate not yet placed, taking gates from
 * the next 256 while the pass keeps at most max_cross_qubits (1..3) qubits >= 4 that branching or
 * swap gates pair keys across; the pass's qubits are the choice, among a few candidates, that
 * takes the most gates. A function of the gates alone (deterministic). SQC_ERR_ARG for a gate
 * invalid on nq qubits. No counterpart in the reference, which applies gates in the order given. */
int sqc_schedule_gates(uint32_t nq, const sqc_gate* gates, uint64_t n, uint32_t max_cross_qubits, uint32_t* perm);
/* Apply one two-qubit gate to a state (the sequence of sqc_twoq_gates). */
int sqc_apply_twoq(sqc_state* st, uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta,
                   double phi, const double* u);

/* Compare two states of equal qubit count on the device (FP64 accumulation):
 * fidelity = |<b|a>|^2 / (<a|a><b|b>), max_abs_err = max over keys of |a_k - b_k|. */
int sqc_compare(sqc_state* a, sqc_state* b, double* fidelity, double* max_abs_err);

/* ---- gate application without allocation ---------------------------------------------- */
/* No counterpart in the reference. For callers that cannot allocate device memory (a host
 * application that owns every device allocation, a plugin limited to the buffers it is
 * handed, code that must not trigger the device-wide synchronization of cudaMalloc/cudaFree):
 * applies n_gates gates (host array, at most 256) to the sparse FP64 state of nq qubits given
 * in the caller's DEVICE arrays keys_in/re_in/im_in (n_in distinct keys, at most 16384) and
 * writes the resulting entries, in no particular order, to the caller's DEVICE arrays
 * keys_out/re_out/im_out (capacity cap_out); *n_out (host) receives their number. Same
 * arithmetic and pair rule as sqc_apply_gates, bit for bit, with the pruning of a state created
 * with the default prune_threshold (1e-14, the only threshold this entry point uses). Keys at or
 * above 2^nq, or given twice, make the call return SQC_ERR_ARG. It calls no
 * cudaMalloc/cudaFree: the table lives in a fixed device array of about 13 MB, held by every
 * device that loads the library until exit. At most 14745 groups of 16 consecutive keys may
 * have been touched during the call (emptied groups included) when a gate pairing keys across
 * groups runs; beyond that, or when *n_out > cap_out, the call returns SQC_ERR_CAPACITY.
 * Calls share the array: serialize calls whose GPU work could overlap. The first call on a
 * device looks up the array's device address and, under CUDA's default lazy module loading,
 * loads the module that holds it (reserving the array, possibly synchronizing): make it during
 * initialisation, before any stream capture, or set CUDA_MODULE_LOADING=EAGER.
 * stream is a cudaStream_t (NULL = default). */
int sqc_apply_fixed(uint32_t nq, const uint64_t* keys_in, const double* re_in, const double* im_in,
                    uint64_t n_in, const sqc_gate* gates, uint64_t n_gates, uint64_t* keys_out,
                    double* re_out, double* im_out, uint64_t cap_out, uint64_t* n_out, void* stream);

/* ---- many-circuit batch ---------------------------------------------------------------- */
/* No counterpart in the reference (one state per process, emulator/device/device_data.cuh:36).
 * A batch runs many independent circuits, each from |0...0>, in one persistent kernel launch:
 * every circuit gets its own table slice, sized from the number of 16-key groups its gates
 * can ever produce (known on the host from which qubits its gates can make differ), so no
 * slice ever grows and the launch needs no host round trip. Each circuit's result is
 * bit-identical to running it alone through sqc_create/sqc_apply_gates. */
typedef struct sqc_batch sqc_batch;

typedef struct sqc_circuit_desc {
    uint32_t nq;              /* qubits, 1..64 */
    uint32_t reserved;
    const sqc_gate* gates;    /* host array, read during sqc_batch_prepare only */
    uint64_t n_gates;
} sqc_circuit_desc;

typedef struct sqc_batch_options {
    uint32_t precision;        /* SQC_FP64 (default) or SQC_FP32 */
    uint32_t device;           /* CUDA device ordinal */
    void* stream;              /* cudaStream_t; NULL = the batch creates its own */
    double prune_threshold;    /* > 0, default 1e-14 */
    double load_factor;        /* groups per bucket of a slice at the group bound, (0, 0.45]; default 0.45 */
    uint32_t min_chunk;        /* list entries a warp takes at once, a multiple of 4; default 8 */
    uint32_t blocks_per_sm;    /* persistent blocks per SM, 0 = as many as fit */
    uint64_t memory_budget;    /* bytes of device memory the batch may hold, 0 = 98% of the device */
    uint32_t use_graph;        /* 1: sqc_batch_run replays a captured CUDA graph */
    uint32_t idle_limit_us;    /* a warp of the persistent kernel that finds no work for this long
                                  ends the run, which then fails with SQC_ERR_STATE (every wait in
                                  the kernel is bounded); 0 = 2 s */
    uint32_t threads_per_unit; /* threads that hold one unit of a pass pairing 16-key groups: 16 (a
                                  pair of groups per half-warp: one qubit >= 4 per pass) or 32 (a
                                  quad per warp: two qubits >= 4 per pass); 0 = 32. Results do not
                                  depend on it; sqc_batch_autotune picks it */
    uint32_t schedule_gates;   /* 1: each circuit is applied in the order sqc_schedule_gates gives it
                                  for two cross-group qubits per pass (whatever threads_per_unit),
                                  as sqc_options.schedule_gates; 0 (default): the order given */
    uint32_t reserved[2];
} sqc_batch_options;

/* Tuning picked by sqc_batch_autotune. */
typedef struct sqc_batch_tuning {
    double load_factor;
    uint32_t min_chunk;
    uint32_t blocks_per_sm;
    double best_ms;            /* run time of the chosen tuning */
    double default_ms;         /* run time of the tuning in effect before the call */
    uint32_t candidates;       /* tunings timed */
    uint32_t threads_per_unit; /* 16 (pair units) or 32 (quad units), see sqc_batch_options */
} sqc_batch_tuning;

typedef struct sqc_batch_stats {
    uint64_t circuits;
    uint64_t passes;           /* passes completed in the last run */
    uint64_t amp_updates;      /* sum over circuits and gates of input nonzeros, last run */
    uint64_t alg_bytes;        /* algorithmic bytes of the passes, last run (sqc_stats.alg_bytes) */
    uint64_t table_bytes;      /* device bytes of the table slices */
    uint64_t kernel_launches;  /* kernels launched by the batch so far */
    double last_run_ms;        /* device time of the last run (CUDA events around its launches) */
} sqc_batch_stats;

void sqc_batch_default_options(sqc_batch_options* opt);
int sqc_batch_create(const sqc_batch_options* opt, sqc_batch** out);
int sqc_batch_destroy(sqc_batch* b);
/* Plan n circuits, lay out their slices and upload their gates. Replaces any earlier circuits.
 * SQC_ERR_BUDGET when the slices do not fit the memory budget. */
int sqc_batch_prepare(sqc_batch* b, const sqc_circuit_desc* circuits, uint32_t n);
/* Run every circuit from |0...0> to its last gate. Asynchronous; may be called repeatedly. */
int sqc_batch_run(sqc_batch* b);
/* Wait for the run. SQC_ERR_STATE if any circuit failed (sqc_batch_circuit_status tells which). */
int sqc_batch_sync(sqc_batch* b);
/* Status of circuit i after sync: SQC_OK, or the error that stopped it. */
int sqc_batch_circuit_status(sqc_batch* b, uint32_t i, int* status);
int sqc_batch_nnz(sqc_batch* b, uint32_t i, uint64_t* nnz);
/* Readout of circuit i, as sqc_get_state. */
int sqc_batch_get_state(sqc_batch* b, uint32_t i, uint64_t* keys, double* re, double* im, uint64_t cap,
                        uint64_t* n, uint32_t flags);
/* Readout of every circuit in one call: circuit i's counts[i] entries follow circuit i-1's in
 * keys/re/im (capacity cap); *total receives the entry count. One readout kernel per circuit
 * and one copy back per array, so the cost is that of the data, not of n round trips. Flags
 * as sqc_get_state (SQC_READ_SORTED orders each circuit's entries). */
int sqc_batch_get_states(sqc_batch* b, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* counts,
                         uint64_t* total, uint32_t flags);
/* Time candidate tunings (load factor, chunk size, blocks per SM) on the prepared circuits and
 * keep the fastest. Runs the batch several times; the circuits' states afterwards are those
 * of a complete run. */
int sqc_batch_autotune(sqc_batch* b, sqc_batch_tuning* out);
int sqc_batch_get_stats(sqc_batch* b, sqc_batch_stats* out);
/* Compare circuit i of a synced batch with a state of the same qubit count, as sqc_compare
 * (fidelity and max |a_k - b_k|, on the device, FP64 accumulation). The state is synced first. */
int sqc_batch_compare(sqc_batch* b, uint32_t i, sqc_state* ref, double* fidelity, double* max_abs_err);
const char* sqc_batch_last_error(sqc_batch* b);
void* sqc_batch_stream(sqc_batch* b);

/* ---- serving loop ---------------------------------------------------------------------- */
/* No counterpart in the reference. Circuits arrive one by one (sqc_server_submit) and are
 * admitted into resident slots while others run: each sqc_server_step admits the queued
 * requests whose table slices fit the memory budget (first come, first served), then runs one
 * time slice of the same persistent kernel as the batch over every resident circuit: circuits
 * that finish leave, the others park at a pass boundary when the slice ends and continue in
 * the next step. States stay on the device between steps and after completion until released.
 * A request's result is bit-identical to running its circuit alone. */
typedef struct sqc_server sqc_server;

typedef struct sqc_server_options {
    uint32_t precision;        /* SQC_FP64 (default) or SQC_FP32 */
    uint32_t device;
    void* stream;              /* cudaStream_t; NULL = the server creates its own */
    double prune_threshold;    /* > 0, default 1e-14 */
    double load_factor;        /* as sqc_batch_options, default 0.45 */
    uint64_t memory_budget;    /* bytes of device memory for slices and gates, 0 = 120 GB (at most 90% of the device) */
    uint32_t max_slots;        /* circuits resident at once, default 1024 */
    uint32_t min_chunk;        /* default 8 */
    double slice_ms;           /* device time of one step before running circuits park, default 2 */
    uint32_t solo_log2_groups; /* circuits that can hold 2^x or more 16-key groups run alone on the
                                  single-state engine (pipelined large-table passes), a slice of
                                  their gates per step; 0 = default (17), 64 = never */
    uint32_t solo_share_pct;   /* percent of the budget kept for those circuits' tables, default 25 */
    uint32_t inject_alloc_failures; /* testing aid for callers' error paths: the next N admissions
                                  (a placement in the pool, or a large circuit's own tables) fail
                                  as an out-of-memory device would: sqc_server_step returns
                                  SQC_ERR_OOM and the request stays queued; 0 (default) = none */
    uint32_t schedule_gates;   /* 1: each circuit is applied in the order sqc_schedule_gates gives it
                                  (three cross-group qubits per pass for large FP32 circuits, else
                                  two), as sqc_options.schedule_gates; 0 (default): the order given */
    uint32_t overlap_steps;    /* 1: sqc_server_step returns once its slice is launched and waits for
                                  it at the next call, so the caller's work between steps (submits,
                                  reads, releases) overlaps the device's; a slice's completions are
                                  reported by the step after it. 0 (default): each step waits for its
                                  own slice */
    uint32_t reserved;
} sqc_server_options;

enum { SQC_REQ_QUEUED = 0, SQC_REQ_RUNNING = 1, SQC_REQ_DONE = 2 };

typedef struct sqc_server_stats {
    uint64_t queued, running, completed;   /* requests in each state (completed: not yet released) */
    uint64_t solo_running;                 /* running requests on the single-state engine */
    uint64_t steps;                        /* steps that launched work */
    uint64_t kernel_launches;
    uint64_t amp_updates;                  /* of the requests completed so far */
    uint64_t pool_bytes, pool_used;        /* the memory budget and its part held by requests (the
                                              tables of up to 16 released large circuits are
                                              kept for the next of the same shape and dropped when
                                              the room is needed; they are not counted here) */
    double busy_ms;                        /* device time of all steps (CUDA events) */
} sqc_server_stats;

void sqc_server_default_options(sqc_server_options* opt);
int sqc_server_create(const sqc_server_options* opt, sqc_server** out);
int sqc_server_destroy(sqc_server* s);
/* Plan a circuit (from |0...0>) and queue it; *id receives the request id. SQC_ERR_BUDGET if
 * the circuit could never fit the memory budget. */
int sqc_server_submit(sqc_server* s, const sqc_circuit_desc* circuit, uint64_t* id);
/* Admit what fits, run one time slice, wait for it (with overlap_steps: wait for the previous
 * step's slice first, then admit and launch this one). *finished (may be NULL) receives the number
 * of requests whose completion the step found. */
int sqc_server_step(sqc_server* s, uint32_t* finished);
/* Ids of completed, unreleased requests (up to cap, oldest first); *n receives their number. */
int sqc_server_completed(sqc_server* s, uint64_t* ids, uint32_t cap, uint32_t* n);
/* state: SQC_REQ_*; status: SQC_OK or the error that stopped the request. */
int sqc_server_request_status(sqc_server* s, uint64_t id, int* state, int* status);
int sqc_server_nnz(sqc_server* s, uint64_t id, uint64_t* nnz);
/* Readout of a completed request, as sqc_get_state. */
int sqc_server_get_state(sqc_server* s, uint64_t id, uint64_t* keys, double* re, double* im, uint64_t cap,
                         uint64_t* n, uint32_t flags);
/* Free the slot and memory of a completed request. */
int sqc_server_release(sqc_server* s, uint64_t id);
int sqc_server_get_stats(sqc_server* s, sqc_server_stats* out);
/* Compare a completed request with a state of the same qubit count, as sqc_compare. */
int sqc_server_compare(sqc_server* s, uint64_t id, sqc_state* ref, double* fidelity, double* max_abs_err);
const char* sqc_server_last_error(sqc_server* s);
void* sqc_server_stream(sqc_server* s);

/* ---- states larger than the device budget ---------------------------------------------
 * The reference's "PC" mode (part of the circuit on one GPU, circuit size > GPU memory;
 * emulator/device/device_data.cuh:20-23), described there but not built. A partitioned state
 * runs in one device table while it fits; when the table cannot grow within device_bytes, the
 * state moves to host memory and the remaining gates run in windows, each partition of the
 * keys (split by qubits >= 4 that the window's non-diagonal gates leave alone) passing through
 * the device table in turn. Results are bit-identical to a single table. Gates are queued;
 * sync, nnz and get_state run them. */
typedef struct sqc_part_state sqc_part_state;

typedef struct sqc_part_stats {
    uint32_t spilled;          /* 1 while the state lives in host memory */
    uint32_t partition_bits;   /* partition qubits of the last window */
    uint64_t spills;           /* moves of the state from the device table to host memory */
    uint64_t returns;          /* moves back to the device table */
    uint64_t windows;          /* gate windows run over host partitions */
    uint64_t bins;             /* partitions run through the device table */
    uint64_t splits;           /* partitions split again because they outgrew the device */
    uint64_t bytes_h2d;        /* state bytes copied host -> device (keys and amplitudes) */
    uint64_t bytes_d2h;        /* state bytes copied device -> host */
    uint64_t amp_updates;      /* sum over gates of input nonzeros, all partitions (after sync) */
    uint64_t max_bin_keys;     /* largest partition loaded into the device table */
    uint64_t table_budget;     /* device bytes the table may use */
} sqc_part_stats;

/* device_bytes: device memory for the working table (0 = the HBM budget of params). opt as for
 * sqc_create (precision, prune threshold, load factor, stream, device). */
int sqc_part_create(uint32_t nq, const sqc_hash_table_parameters* params, const sqc_options* opt,
                    uint64_t device_bytes, sqc_part_state** out);
int sqc_part_destroy(sqc_part_state* st);
int sqc_part_set_zero_state(sqc_part_state* st);
int sqc_part_apply_gates(sqc_part_state* st, const sqc_gate* gates, uint64_t n);
int sqc_part_sync(sqc_part_state* st);
int sqc_part_nnz(sqc_part_state* st, uint64_t* n);
/* As sqc_get_state (flags SQC_READ_SORTED, SQC_READ_DROP_NEGLIGIBLE). */
int sqc_part_get_state(sqc_part_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, uint64_t* n_out,
                       uint32_t flags);
int sqc_part_get_stats(sqc_part_state* st, sqc_part_stats* out);
const char* sqc_part_last_error(sqc_part_state* st);

/* ---- introspection ------------------------------------------------------------------- */
typedef struct sqc_stats {
    uint64_t gates_applied;    /* gates executed on the device */
    uint64_t passes;           /* device gate passes executed */
    uint64_t kernel_launches;  /* kernels launched by this handle */
    uint64_t buckets;          /* current buckets per table */
    uint64_t table_bytes;      /* device bytes held by both tables */
    uint64_t replays;          /* passes re-run after table growth */
    uint64_t amp_updates;      /* sum over gates of input nonzeros (only counted after sync) */
    uint64_t alg_bytes;        /* algorithmic bytes of the passes: (nnz_in + nnz_out) * (8 + A) per
                                  key-changing pass, nnz * (8 + 2A) per pass that keeps every key;
                                  A = 16 (FP64) or 8 (FP32). Since the last reset, after sync. */
    uint64_t alg_bytes_pair;   /* the part of alg_bytes moved by pair passes (a gate pairing keys of
                                  different 16-key groups, plus the gates fused after it) */
    uint64_t passes_pair;      /* pair passes among `passes` */
    uint64_t pass_ns_pair;     /* device time of the pair passes, from CUDA events (time_passes = 1;
                                  since creation, after sync) */
    uint64_t pass_ns_stream;   /* device time of the other passes, likewise */
} sqc_stats;

int sqc_get_stats(sqc_state* st, sqc_stats* out);
/* Device diagnostic (no counterpart in the reference): the FP64 fused multiply-add rate of
 * device `device`, in lane operations per second, from a timed loop of independent FMA chains
 * (synchronizes the device; allocates 8 bytes for the duration of the call). On this GPU the
 * FP64 pipe bounds the FP64 gate passes, and this is its measured peak. */
int sqc_fp64_rate(uint32_t device, double* fma_per_s);
const char* sqc_status_string(int status);
/* Message of the last error on this handle ("" if none). Valid until the next call. */
const char* sqc_last_error(sqc_state* st);
/* The cudaStream_t the handle runs on. */
void* sqc_stream(sqc_state* st);

#ifdef __cplusplus
}
#endif
#endif /* SPARQC_H */
