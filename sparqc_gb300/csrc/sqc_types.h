// Plain data structures shared by the host engine and the kernels (no device code).
#pragma once
#include <cstdint>

namespace sqc {

constexpr int kSlots = 16;
constexpr int kSlotBits = 4;
constexpr uint32_t kMaxProbe = 256;   // buckets probed before a claim reports the table full
constexpr int kThreads = 256;
constexpr int kMaxRun = 64;           // gates fused into one pass at most
constexpr unsigned kFull = 0xffffffffu;

enum Status : unsigned int { ST_OK = 0, ST_TABLE_FULL = 1, ST_DUPLICATE = 2 };

// gate kinds (same numbering as sqc_gate.kind)
enum Kind : uint32_t { KX = 0, KY, KZ, KH, KPHASE, KRZ, KRX, KRY, KS, KSDG, KT, KTDG, KU, KCOUNT };

struct alignas(16) Header {
    unsigned long long group;
    unsigned int epoch;
    unsigned int aux;
};

struct TableDev {
    Header* hdr;
    unsigned long long* keys;
    void* amps;
    unsigned long long mask;   // nb - 1
};

// Device-resident control block of one state. All per-pass bookkeeping happens here, on the
// device, so a recorded sequence of passes can be replayed without host involvement.
struct Ctl {
    unsigned int epoch[2];     // epoch of each table's current content
    unsigned int status;       // Status; nonzero stops every later pass until the host repairs
    unsigned int done;         // blocks finished in the running pass
    unsigned long long seq;    // passes completed since the last reset
    unsigned long long nnz[2];     // keys held by each table's content
    unsigned long long groups[2];  // live buckets of each table's content
    unsigned long long acc_nnz, acc_groups, acc_upd;
    unsigned long long amp_updates;  // sum over gates of input nonzeros, since the last reset
    unsigned long long alg_bytes;    // algorithmic bytes of the passes, since the last reset
    unsigned long long out_count;    // readout / set-state counter
    double acc[6];                   // reductions: norm, compare
    unsigned long long acc_max;      // bit pattern of a non-negative double (max |a-b|)
};

// Gate descriptor with host-resolved coefficients (std::cos/std::sin on the host, so the
// device and the CPU oracle use identical values).
struct GateDesc {
    uint32_t kind, target;
    unsigned long long ctrl;
    double c, s;          // phase/T/Tdg: cos, sin; rz/rx/ry: cos, sin of theta/2; h: 1/sqrt(2)
    double m[8];          // u: m00, m01, m10, m11 as (re, im)
    float cf, sf;         // float copies for FP32 states
    float mf[8];
};

struct PruneBits {
    unsigned long long d;   // bit pattern of thr (double)
    unsigned int f;         // bit pattern of the largest float below thr
};

struct PassArgs {
    TableDev tab[2];
    Ctl* ctl;
    const GateDesc* gates;
    uint32_t g0, g1;      // gate range [g0, g1) of this pass
    uint32_t parity;      // input table index
    uint32_t pair;        // 1: first gate pairs groups G and G ^ (1 << (target - 4))
    uint32_t keys_fixed;  // 1: every gate of the pass is diagonal (no key changes)
    uint32_t amp_bytes;   // 16 (FP64) or 8 (FP32)
    PruneBits prune;
};

}  // namespace sqc
