// Plain data structures shared by the host engine and the kernels (no device code).
#pragma once
#include <cstdint>

namespace sqc {

constexpr int kSlots = 16;
constexpr int kSlotBits = 4;
constexpr uint32_t kMaxProbe = 4096;  // buckets probed before a claim reports the table full
constexpr int kThreads = 256;
constexpr int kMaxRun = 64;           // gates fused into one pass at most
constexpr unsigned kFull = 0xffffffffu;

enum Status : unsigned int {
    ST_OK = 0,
    ST_TABLE_FULL = 1,   // a claim found no free bucket within kMaxProbe (state no longer valid)
    ST_DUPLICATE = 2,    // set_state saw the same key twice
    ST_GROW = 3,         // a pair pass refused to start: the table might overflow (state intact)
    ST_TIMEOUT = 4,      // a bounded wait inside a pass ran out (state no longer valid)
    ST_BAD_KEY = 5       // a loaded key has a bit at or above the register's qubit count
};

// gate kinds (0..12 = sqc_gate.kind); KYPH is internal: the diagonal left over when an
// uncontrolled Y is turned into a relabelling of the keys (bit 0 -> -i, bit 1 -> +i).
enum Kind : uint32_t { KX = 0, KY, KZ, KH, KPHASE, KRZ, KRX, KRY, KS, KSDG, KT, KTDG, KU, KCOUNT, KYPH = 13 };

struct alignas(16) Header {
    unsigned long long group;   // key >> 4 of the bucket's keys
    unsigned int epoch;         // live iff equal to the state's epoch
    unsigned int aux;           // 0
};

// One unit of a pass that pairs groups, resolved before the pass. With cross-group qubits
// q1, q2, q3 (masks m1 = 1 << (q1 - 4), ...; a pair pass has q1 only, a quad pass q1 and q2),
// the unit is the set of groups G0 | i0*m1 | i1*m2 | i2*m3 with G0 having those stored bits 0;
// b[i0 + 2*i1 + 4*i2] is the bucket of member (i0, i1, i2), kNoBucket when the group is absent.
// Pair passes use b[0..1], quad passes b[0..3], octet passes b[0..7].
constexpr unsigned kNoBucket = 0xFFFFFFFFu;
struct alignas(16) Unit {
    unsigned long long G0;
    unsigned int b[8];
};

struct TableDev {
    Header* hdr;
    unsigned long long* keys;
    void* amps;
    unsigned int* list;         // live buckets, in claim order
    Unit* units;                // owned units of a pair or quad pass, compacted by the resolve kernel
    unsigned long long mask;    // nb - 1
};

// Device-resident control block of one state. Per-pass bookkeeping happens here, on the
// device, so a recorded sequence of passes replays without host involvement.
struct Ctl {
    unsigned int epoch;             // live-bucket epoch of the table
    unsigned int status;            // Status; nonzero stops every later pass until the host repairs
    unsigned int done;              // blocks finished in the running pass
    unsigned int pad0;
    unsigned long long seq;         // passes completed since the last reset
    unsigned long long nnz;         // keys held
    unsigned long long list_n;      // live buckets (list entries) committed at the last pass end
    unsigned long long list_tail;   // list entries appended so far
    unsigned long long empty_groups;  // live buckets without a key after the last pass
    unsigned long long acc_nnz, acc_upd, acc_empty;
    unsigned long long amp_updates; // sum over gates of input nonzeros, since the last reset
    unsigned long long alg_bytes;   // algorithmic bytes of the passes, since the last reset
    unsigned long long alg_bytes_pair;  // the part of alg_bytes moved by pair passes
    unsigned long long out_count;   // readout counter
    double acc[6];                  // reductions: norm, compare
    unsigned long long acc_max;     // bit pattern of a non-negative double (max |a-b|)
    unsigned long long work;        // list entries handed out in the running pass (0 between passes)
    unsigned long long units_n;     // owned units the running pass's resolve kernel wrote (0 between passes)
};

// Gate descriptor with host-resolved coefficients (std::cos/std::sin on the host, so the
// device and the CPU oracle use identical values) in the stored-key frame: the gate acts on
// a stored key s iff (s & ctrl) == cval, and the member's logical target bit is
// ((s >> target) & 1) ^ flip. The first 32 bytes (kind .. pad) are read as two 16-byte
// vectors, hence the alignment. `flip` holds the frame flip in bit 0 and, once the gate's
// pass is known, how that pass applies it (kOp* bits, set by encode_pass on the host).
struct alignas(16) GateDesc {
    uint32_t kind, target;
    unsigned long long ctrl, cval;
    uint32_t flip, pad;
    double c, s;          // phase/T/Tdg: cos, sin; rz/rx/ry: cos, sin of theta/2; h: 1/sqrt(2)
    double m[8];          // u: m00, m01, m10, m11 as (re, im)
    float cf, sf;         // float copies for FP32 states
    float mf[8];
};

// GateDesc.flip bits.
constexpr uint32_t kOpFlip = 1u << 0;      // the stored frame flips the target bit
constexpr uint32_t kOpPair = 1u << 1;      // pairs the a and b slots (first cross-group qubit)
constexpr uint32_t kOpShfl = 1u << 2;      // partner slot in lane ^ (1 << off_log2)
constexpr uint32_t kOpOffShift = 3;        // off_log2: bits 3..5
constexpr uint32_t kOpCtrl = 1u << 6;      // controls to test per key
constexpr uint32_t kOpBranch = 1u << 7;    // H, Rx, Ry, U
constexpr uint32_t kOpSwap = 1u << 8;      // X, Y
constexpr uint32_t kOpOneSided = 1u << 9;  // diagonal gate that leaves bit-0 keys unchanged
constexpr uint32_t kOpLowBit = 1u << 10;   // target < 4: the target bit is in the slot index
constexpr uint32_t kOpPair3 = 1u << 11;    // pairs slots a with c and b with d (third cross-group qubit)

struct PruneBits {
    unsigned long long d;   // bit pattern of thr (double)
    unsigned int f;         // bit pattern of the largest float below thr
};

constexpr uint32_t kNoQubit = 0xFFFFFFFFu;

// Exact sums of products (sqc_exact.cuh): fixed-point numbers with their least significant bit
// at 2^kSumLsb, kSumChunks 32-bit pieces each held in a 64-bit counter.
constexpr int kSumChunks = 10;
constexpr int kSumLsb = -256;
enum SumIndex { SUM_NORM = 0, SUM_ORE, SUM_OIM, SUM_NA, SUM_NB, SUM_NB_ONLY, kSums };
struct ExactSums {
    unsigned long long c[kSums][kSumChunks];
};

// One pass of a single-launch run over a tiny table (tiny_kernel): what PassArgs says per pass.
struct TinyPass {
    uint32_t g0, g1, nx, q1, q2, q3, keys_fixed, pad;
    unsigned long long grow_bound;
};

struct PassArgs {
    TableDev t;
    Ctl* ctl;
    const GateDesc* gates;
    uint32_t g0, g1;        // gate range [g0, g1) of this pass
    uint32_t nx;            // cross-group qubits of the pass: 0 (stream), 1 (pair) or 2 (quad)
    uint32_t keys_fixed;    // 1: every gate of the pass is diagonal (no key changes)
    uint32_t amp_bytes;     // 16 (FP64) or 8 (FP32)
    uint32_t credit;        // gates resolved on the host just before this pass (identity or
                            // relabel): each is credited with this pass's input key count
    unsigned long long max_groups;   // a pass that pairs groups refuses to start when its groups
                                     // could exceed this: min(grow_bound, n << nx) > max_groups
    PruneBits prune;
    uint32_t q1, q2, q3;             // the cross-group qubits (kNoQubit when absent)
    unsigned long long grow_bound;   // groups the state can hold after the pass, at most
};

}  // namespace sqc
