// sqc_apply_fixed: gate application that allocates nothing.
//
// Some callers cannot allocate device memory: a host application that owns every device
// allocation through its own arena, a plugin that may only use the buffers it is handed, or
// code running where an allocation would stall or fail (for example while other work on the
// device must not be disturbed by a cudaMalloc/cudaFree, which synchronizes the device).
// This entry point serves them. The caller passes its sparse state and receives the result
// in device arrays it owns; the hash table, its control block and the gate descriptors live
// in one file-scope device array of fixed size, held by every device that loads it until the
// process exits. With CUDA's lazy module loading (the default) the module holding the array is
// loaded on a device by the first call made there, which then reserves the array (about 13 MB)
// and may synchronize: make that first call during initialisation, or load modules eagerly
// (CUDA_MODULE_LOADING=EAGER).
//
// Pruning uses the engine's default threshold, 1e-14: results equal sqc_apply_gates' for states
// created with the default prune_threshold. Input keys must lie below 2^nq and be distinct
// (SQC_ERR_ARG otherwise).
// Limits: FP64 amplitudes; at most kFixedMaxInput input keys and kFixedMaxGates gates per
// call; at most 14745 (= 0.45 * kFixedBuckets) groups of 16 consecutive keys may have been
// touched when a gate that pairs keys across groups runs (branching or X/Y gates on qubits
// >= 4) -- 235,920 keys when the groups are full. A group emptied during the call (all its
// keys pruned or moved away) still counts: only the allocating path compacts the table.
// Larger inputs are rejected up front; a state that outgrows the table during the call ends
// the call with SQC_ERR_CAPACITY.
//
// Every call uses the same array and leaves its contents behind; the control block is reset
// at the start of each call and stale buckets are told apart by an epoch. Calls whose GPU
// work overlaps (different streams, or different host threads without ordering) race on
// the array: serialize them. The device address of the array is looked up once per device
// (cudaGetSymbolAddress, with that device current) on the first call made on it; make that
// first call before any stream capture.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/sparqc.h"
#include "sqc_kernels.h"
#include "sqc_plan.h"

namespace sqc {
namespace {

constexpr unsigned long long kFixedBuckets = 1ULL << 15;
constexpr unsigned long long kFixedMaxInput = 1ULL << 14;
constexpr unsigned long long kFixedMaxGates = 256;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffHdr = 0;
constexpr size_t kOffKeys = align256(kOffHdr + kFixedBuckets * sizeof(Header));
constexpr size_t kOffAmps = align256(kOffKeys + kFixedBuckets * kSlots * sizeof(unsigned long long));
constexpr size_t kOffList = align256(kOffAmps + kFixedBuckets * kSlots * 16);
constexpr size_t kOffCtl = align256(kOffList + kFixedBuckets * sizeof(unsigned));
constexpr size_t kOffDesc = align256(kOffCtl + sizeof(Ctl));
constexpr size_t kScratchBytes = align256(kOffDesc + kFixedMaxGates * sizeof(GateDesc));

// The scratch of every call (about 13 MB). Host code must not use this name as an address.
static __device__ __align__(256) unsigned char g_fixed_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_fixed_mu;
void* g_fixed_base[kMaxDevices] = {};
int g_fixed_sms[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t fixed_base(int dev, void** out, int* sms) {
    std::lock_guard<std::mutex> lock(g_fixed_mu);
    if (!g_fixed_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scratch);
        if (e != cudaSuccess) return e;
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        g_fixed_base[dev] = p;
        g_fixed_sms[dev] = n;
    }
    *out = g_fixed_base[dev];
    *sms = g_fixed_sms[dev];
    return cudaSuccess;
}

bool diag_kind(uint32_t k) { return k == KZ || k == KPHASE || k == KRZ || k == KS || k == KSDG || k == KT || k == KTDG; }

// Keys with a bit at or above nq are not states of the register: flag them (ST_BAD_KEY).
__global__ void fixed_key_check_kernel(const unsigned long long* __restrict__ keys, unsigned long long n,
                                       unsigned long long outside, Ctl* ctl) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        if (keys[i] & outside) atomicCAS(&ctl->status, 0u, (unsigned)ST_BAD_KEY);
}

// Calls made on each device since its scratch headers were last cleared. Every call bumps the
// table epoch once; before the 32-bit epoch could come back to a value stale headers hold, the
// headers and the control block are cleared (cudaMemsetAsync allocates nothing).
unsigned long long g_fixed_calls[kMaxDevices] = {};
constexpr unsigned long long kEpochRestart = 0xFFFFFF00ULL;

}  // namespace
}  // namespace sqc

extern "C" int sqc_apply_fixed(uint32_t nq, const uint64_t* keys_in, const double* re_in, const double* im_in,
                               uint64_t n_in, const sqc_gate* gates, uint64_t n_gates, uint64_t* keys_out,
                               double* re_out, double* im_out, uint64_t cap_out, uint64_t* n_out, void* stream) {
    using namespace sqc;
    if (nq < 1 || nq > 64 || !n_out) return SQC_ERR_ARG;
    *n_out = 0;
    if (n_in > kFixedMaxInput || n_gates > kFixedMaxGates) return SQC_ERR_CAPACITY;
    if (n_in && (!keys_in || !re_in || !im_in)) return SQC_ERR_ARG;
    if (n_gates && !gates) return SQC_ERR_ARG;
    if (cap_out && (!keys_out || !re_out || !im_out)) return SQC_ERR_ARG;
    GateDesc hd[kFixedMaxGates];
    for (uint64_t i = 0; i < n_gates; ++i) {
        const sqc_gate& g = gates[i];
        if (check_gate(g, nq)) return SQC_ERR_ARG;
        hd[i] = make_desc(Planner{}, g.kind, g.target, g.controls, g);   // identity key frame
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SQC_ERR_NO_DEVICE;
    void* base = nullptr;
    int sms = 1;
    if (fixed_base(dev, &base, &sms) != cudaSuccess) return SQC_ERR_CUDA;
    unsigned char* b = static_cast<unsigned char*>(base);
    TableDev t;
    t.hdr = reinterpret_cast<Header*>(b + kOffHdr);
    t.keys = reinterpret_cast<unsigned long long*>(b + kOffKeys);
    t.amps = b + kOffAmps;
    t.list = reinterpret_cast<unsigned*>(b + kOffList);
    t.units = nullptr;    // small tables take the direct pass, which needs neither
    t.mask = kFixedBuckets - 1;
    Ctl* ctl = reinterpret_cast<Ctl*>(b + kOffCtl);
    GateDesc* d_desc = reinterpret_cast<GateDesc*>(b + kOffDesc);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    {
        std::lock_guard<std::mutex> lock(g_fixed_mu);
        if (++g_fixed_calls[dev] >= kEpochRestart) {
            if (cudaMemsetAsync(t.hdr, 0, kFixedBuckets * sizeof(Header), st) != cudaSuccess ||
                cudaMemsetAsync(ctl, 0, sizeof(Ctl), st) != cudaSuccess)
                return SQC_ERR_CUDA;
            g_fixed_calls[dev] = 1;
        }
    }
    // load the caller's state (the kernels read its device arrays; the epoch bump frees the table)
    if (launch_set_state(reinterpret_cast<const unsigned long long*>(keys_in), re_in, im_in, n_in, t, ctl, true,
                         sms, st) != cudaSuccess)
        return SQC_ERR_CUDA;
    if (nq < 64 && n_in) {
        const unsigned long long outside = ~((1ULL << nq) - 1);
        const int grid = (int)std::min<unsigned long long>((n_in + 255) / 256, (unsigned long long)sms * 4);
        fixed_key_check_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<const unsigned long long*>(keys_in), n_in,
                                                     outside, ctl);
        if (cudaGetLastError() != cudaSuccess) return SQC_ERR_CUDA;
    }
    // same pass split as the engine with one cross-group qubit per pass: one cross-group gate,
    // then a stream run; each pass's gates are encoded before the descriptors are uploaded
    struct Span {
        uint32_t g0, g1, q1;
        bool pair, fixed;
    };
    Span spans[kFixedMaxGates];
    size_t ns = 0, i = 0;
    while (i < n_gates) {
        const size_t start = i;
        auto streamable = [&](size_t k) { return hd[k].target < (uint32_t)kSlotBits || diag_kind(hd[k].kind); };
        const bool pair = !streamable(i);
        if (pair) ++i;
        while (i < n_gates && i - start < (size_t)kMaxRun && streamable(i)) ++i;
        bool fixed = true;
        for (size_t k = start; k < i; ++k) fixed = fixed && diag_kind(hd[k].kind);
        const uint32_t q1 = pair ? hd[start].target : kNoQubit;
        encode_pass(hd, start, i, q1);
        spans[ns++] = Span{(uint32_t)start, (uint32_t)i, q1, pair, fixed};
    }
    if (n_gates && cudaMemcpyAsync(d_desc, hd, n_gates * sizeof(GateDesc), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return SQC_ERR_CUDA;

    PassArgs a;
    std::memset(&a, 0, sizeof a);
    a.t = t;
    a.ctl = ctl;
    a.gates = d_desc;
    a.amp_bytes = 16;
    a.max_groups = (unsigned long long)(0.9 * (double)kFixedBuckets);
    const double thr = 1e-14;
    std::memcpy(&a.prune.d, &thr, sizeof(double));
    float tf = (float)thr;
    if ((double)tf >= thr) tf = std::nextafter(tf, 0.0f);
    std::memcpy(&a.prune.f, &tf, sizeof(float));
    for (size_t k = 0; k < ns; ++k) {
        a.g0 = spans[k].g0;
        a.g1 = spans[k].g1;
        a.nx = spans[k].pair ? 1u : 0u;
        a.q1 = spans[k].q1;
        a.q2 = kNoQubit;
        a.q3 = kNoQubit;
        a.grow_bound = ~0ULL;
        a.keys_fixed = spans[k].fixed ? 1u : 0u;
        if (launch_pass(a, kFixedBuckets, true, sms, st) < 0) return SQC_ERR_CUDA;
    }
    if (launch_readout(t, ctl, kFixedBuckets, 0ULL, true, reinterpret_cast<unsigned long long*>(keys_out), re_out,
                       im_out, cap_out, false, a.prune, sms, st) != cudaSuccess)
        return SQC_ERR_CUDA;
    Ctl c;
    if (cudaMemcpyAsync(&c, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st) != cudaSuccess) return SQC_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SQC_ERR_CUDA;
    if (c.status == ST_GROW || c.status == ST_TABLE_FULL) return SQC_ERR_CAPACITY;
    if (c.status == ST_DUPLICATE || c.status == ST_BAD_KEY) return SQC_ERR_ARG;
    if (c.status != ST_OK) return SQC_ERR_STATE;
    *n_out = c.out_count;
    return c.out_count > cap_out ? SQC_ERR_CAPACITY : SQC_OK;
}
