// Device-side layout and arithmetic of the sparse statevector table.
//
// Table layout (one table per state, updated in place by every pass):
//   hdr [nb]          16-byte bucket headers {group, epoch, aux}
//   keys[nb * 16]     64-bit stored keys, 16 per bucket (128 bytes)
//   amps[nb * 16]     amplitudes, double2 (FP64) or float2 (FP32), same slot order
//   list[nb]          indices of the live buckets, in claim order
// A bucket holds the keys of one group G = key >> 4 at slot key & 15. Buckets are found by
// linear probing from mix(G) & (nb - 1). A bucket is live iff hdr.epoch equals the state's
// epoch, so a reset only bumps the epoch. A slot is occupied iff the low 4 bits of its
// stored key equal the slot index; empty slots hold EMPTY(j) = 0xFFFF...F0 | (15 - j).
// Live buckets are never freed between resets: a group whose keys are all pruned stays as an
// empty live bucket, so probe chains never break.
//
// The reference keeps one dense slot per basis state (identity hash, 2^nq slots,
// emulator/device/table_manager.cuh:114-119, emulator/include/sim_parameters_types.h:153-158);
// here the table is sized by load factor and holds only present keys, so 64-qubit keys work.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "sqc_types.h"

namespace sqc {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31; return x;
}

__device__ __forceinline__ unsigned long long empty_key(int j) {
    return 0xFFFFFFFFFFFFFFF0ULL | (unsigned long long)(15 - j);
}

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
    unsigned lo = __shfl_sync(kFull, (unsigned)v, src);
    unsigned hi = __shfl_sync(kFull, (unsigned)(v >> 32), src);
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ Header load_hdr(const Header* p) {
    ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
    Header h;
    h.group = v.x;
    h.epoch = (unsigned)v.y;
    h.aux = (unsigned)(v.y >> 32);
    return h;
}

__device__ __forceinline__ Header load_hdr_cg(const Header* p) {
    ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2*>(p));
    Header h;
    h.group = v.x;
    h.epoch = (unsigned)v.y;
    h.aux = (unsigned)(v.y >> 32);
    return h;
}

// 128-bit compare-and-swap on a bucket header. Returns the previous content.
__device__ __forceinline__ Header cas_hdr(Header* p, const Header& expect, const Header& desired) {
    unsigned long long e0 = expect.group, e1 = (unsigned long long)expect.epoch | ((unsigned long long)expect.aux << 32);
    unsigned long long d0 = desired.group, d1 = (unsigned long long)desired.epoch | ((unsigned long long)desired.aux << 32);
    unsigned long long o0, o1;
    asm volatile(
        "{\n\t.reg .b128 d, c, s;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 s, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, s;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(o0), "=l"(o1)
        : "l"(e0), "l"(e1), "l"(d0), "l"(d1), "l"(p)
        : "memory");
    Header o;
    o.group = o0;
    o.epoch = (unsigned)o1;
    o.aux = (unsigned)(o1 >> 32);
    return o;
}

// Find the live bucket of group G, or -1. Correct while other threads claim buckets: a
// claim only turns a non-live bucket live, and G's probe chain has no non-live bucket.
__device__ __forceinline__ long long lookup_group(const TableDev& t, unsigned ep, unsigned long long G) {
    unsigned long long b = mix64(G) & t.mask;
    for (uint32_t i = 0; i < kMaxProbe; ++i) {
        const Header h = load_hdr_cg(t.hdr + b);
        if (h.epoch != ep) return -1;
        if (h.group == G) return (long long)b;
        b = (b + 1) & t.mask;
    }
    return -1;
}

// Claim (or find) the bucket of group G: linear probing with a 128-bit CAS per attempt,
// bounded. *created tells whether this call turned the bucket live. -1 and ST_TABLE_FULL
// when no bucket within kMaxProbe of the home bucket is free.
__device__ __forceinline__ long long claim_group(const TableDev& t, unsigned ep, unsigned long long G,
                                                 unsigned int* status, bool* created) {
    *created = false;
    unsigned long long b = mix64(G) & t.mask;
    Header cur = load_hdr_cg(t.hdr + b);
    uint32_t probes = 0, attempts = 0;
    while (probes < kMaxProbe && attempts < 4 * kMaxProbe) {
        ++attempts;
        if (cur.epoch == ep) {
            if (cur.group == G) return (long long)b;
            b = (b + 1) & t.mask;
            ++probes;
            cur = load_hdr_cg(t.hdr + b);
            continue;
        }
        Header want;
        want.group = G; want.epoch = ep; want.aux = 0;
        const Header old = cas_hdr(t.hdr + b, cur, want);
        if (old.group == cur.group && old.epoch == cur.epoch && old.aux == cur.aux) {
            *created = true;
            return (long long)b;
        }
        cur = old;   // re-examine this bucket with its actual content
    }
    atomicCAS(status, 0u, (unsigned)ST_TABLE_FULL);
    return -1;
}

// ---- arithmetic --------------------------------------------------------------------------
// Explicit round-to-nearest operations: nothing is contracted, so every product and sum
// rounds exactly as in the reference's source formulas (emulator/device/device_data.cuh:159-319).
template <class T> struct Arith;
template <> struct Arith<double> {
    __device__ static __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ static __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
};
template <> struct Arith<float> {
    __device__ static __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ static __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ static __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};

template <class T> struct Cx { T r, i; };

// Sign flips and magnitude tests as integer operations: on this GPU every FP64 instruction,
// compares and negations included, issues on the slow FP64 pipe. Both forms are exact. The
// flip is an opaque integer xor on the high word, so the compiler cannot turn it back into
// a floating-point negation (which it may lower to an FP64 add).
__device__ __forceinline__ double neg(double x) {
    int hi = __double2hiint(x);
    const int lo = __double2loint(x);
    asm("xor.b32 %0, %0, 0x80000000;" : "+r"(hi));
    return __hiloint2double(hi, lo);
}
__device__ __forceinline__ float neg(float x) {
    int v = __float_as_int(x);
    asm("xor.b32 %0, %0, 0x80000000;" : "+r"(v));
    return __int_as_float(v);
}

// Gate descriptors are read-only for a whole launch and read by every warp for every slot it
// holds, while the table streams through the same L1: the pass kernels mark descriptor loads
// to stay in L1 (evict_last), so the table's traffic does not push them out to L2 between
// uses. The persistent batch kernel, whose loads default to L2 only, keeps the plain
// non-coherent loads (SQC_DESC_EVICT_LAST 0), which measured faster there.
#ifndef SQC_DESC_EVICT_LAST
#define SQC_DESC_EVICT_LAST 1
#endif
__device__ __forceinline__ uint4 ld_desc4(const void* p) {
#if SQC_DESC_EVICT_LAST
    uint4 v;
    asm("ld.global.nc.L1::evict_last.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
#else
    return __ldg(reinterpret_cast<const uint4*>(p));
#endif
}
__device__ __forceinline__ double ld_desc(const double* p) {
#if SQC_DESC_EVICT_LAST
    double v;
    asm("ld.global.nc.L1::evict_last.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}
__device__ __forceinline__ float ld_desc(const float* p) {
#if SQC_DESC_EVICT_LAST
    float v;
    asm("ld.global.nc.L1::evict_last.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}

// Programmatic dependent launch. Direct passes are launched with programmatic stream
// serialization, so the next pass's blocks may be placed on the SMs while the running pass
// drains. Such a kernel first waits until the previous grid in the stream has completed and
// its writes are visible (a no-op without that launch attribute), and then lets the next pass
// be scheduled: its blocks only wait in turn, and all of this grid's blocks are already
// resident by then, so nothing waits on a block that cannot be placed.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// A gate's (c, s) pair copied to shared memory, with its descriptor for the U matrix.
template <class T> struct SmemCoef {
    T c, s;
    const GateDesc* g;
};

// Coefficients are read through a pointer to the (L1-resident, warp-broadcast) descriptor, or
// from the pair a pass staged in shared memory.
template <class T> struct Coef;
template <> struct Coef<double> {
    __device__ static __forceinline__ double c(const GateDesc* g) { return ld_desc(&g->c); }
    __device__ static __forceinline__ double s(const GateDesc* g) { return ld_desc(&g->s); }
    __device__ static __forceinline__ double m(const GateDesc* g, int i) { return ld_desc(&g->m[i]); }
    __device__ static __forceinline__ double c(const SmemCoef<double>& k) { return k.c; }
    __device__ static __forceinline__ double s(const SmemCoef<double>& k) { return k.s; }
    __device__ static __forceinline__ double m(const SmemCoef<double>& k, int i) { return ld_desc(&k.g->m[i]); }
};
template <> struct Coef<float> {
    __device__ static __forceinline__ float c(const GateDesc* g) { return ld_desc(&g->cf); }
    __device__ static __forceinline__ float s(const GateDesc* g) { return ld_desc(&g->sf); }
    __device__ static __forceinline__ float m(const GateDesc* g, int i) { return ld_desc(&g->mf[i]); }
    __device__ static __forceinline__ float c(const SmemCoef<float>& k) { return k.c; }
    __device__ static __forceinline__ float s(const SmemCoef<float>& k) { return k.s; }
    __device__ static __forceinline__ float m(const SmemCoef<float>& k, int i) { return ld_desc(&k.g->mf[i]); }
};

// Branching update seen from one member of a pair, for gate kind K: a = own amplitude,
// b = partner amplitude, bit = own logical target bit. Each form rounds exactly like the
// reference's pair formula for that member (a + (-b) == a - b and (-s)*x == -(s*x) hold
// exactly in IEEE arithmetic):
//   H : bit 0 -> f*(v0 + v1),             bit 1 -> f*(v0 - v1)
//   Rx: c*own + s*(i-rotated partner)      (symmetric in the two members)
//   Ry: bit 0 -> c*v0 - s*v1,             bit 1 -> c*v1 + s*v0
//   U : self term first, then partner term, fused multiply-add chain (no reference form).
template <class T, uint32_t K, class G>
__device__ __forceinline__ Cx<T> branch_update(const G& g, bool bit, Cx<T> a, Cx<T> b) {
    using A = Arith<T>;
    Cx<T> o;
    if constexpr (K == KH) {
        const T f = Coef<T>::c(g);
        const Cx<T> x = bit ? b : a;
        const Cx<T> y = bit ? Cx<T>{neg(a.r), neg(a.i)} : b;
        o.r = A::mul(f, A::add(x.r, y.r));
        o.i = A::mul(f, A::add(x.i, y.i));
    } else if constexpr (K == KRX) {
        const T c = Coef<T>::c(g), s = Coef<T>::s(g);
        o.r = A::add(A::mul(c, a.r), A::mul(s, b.i));
        o.i = A::sub(A::mul(c, a.i), A::mul(s, b.r));
    } else if constexpr (K == KRY) {
        const T c = Coef<T>::c(g), s0 = Coef<T>::s(g);
        const T s = bit ? s0 : neg(s0);
        o.r = A::add(A::mul(c, a.r), A::mul(s, b.r));
        o.i = A::add(A::mul(c, a.i), A::mul(s, b.i));
    } else {  // KU
        const T m00r = Coef<T>::m(g, 0), m00i = Coef<T>::m(g, 1), m01r = Coef<T>::m(g, 2), m01i = Coef<T>::m(g, 3);
        const T m10r = Coef<T>::m(g, 4), m10i = Coef<T>::m(g, 5), m11r = Coef<T>::m(g, 6), m11i = Coef<T>::m(g, 7);
        const T msr = bit ? m11r : m00r, msi = bit ? m11i : m00i;
        const T mor = bit ? m10r : m01r, moi = bit ? m10i : m01i;
        o.r = A::fma(neg(moi), b.i, A::fma(mor, b.r, A::fma(neg(msi), a.i, A::mul(msr, a.r))));
        o.i = A::fma(moi, b.r, A::fma(mor, b.i, A::fma(msi, a.r, A::mul(msr, a.i))));
    }
    return o;
}

// Diagonal update of one amplitude for gate kind K (reference: z_core, phase_core, rz_core).
template <class T, uint32_t K, class G>
__device__ __forceinline__ Cx<T> diag_update(const G& g, bool bit, Cx<T> a) {
    using A = Arith<T>;
    if constexpr (K == KZ) return bit ? Cx<T>{neg(a.r), neg(a.i)} : a;
    else if constexpr (K == KS) return bit ? Cx<T>{neg(a.i), a.r} : a;
    else if constexpr (K == KSDG) return bit ? Cx<T>{a.i, neg(a.r)} : a;
    else if constexpr (K == KYPH) return bit ? Cx<T>{neg(a.i), a.r} : Cx<T>{a.i, neg(a.r)};
    else if constexpr (K == KRZ) {
        const T c = Coef<T>::c(g), s0 = Coef<T>::s(g);
        const T s = bit ? s0 : neg(s0);   // bit 0: conj(a)*v0, bit 1: a*v1
        return Cx<T>{A::sub(A::mul(c, a.r), A::mul(s, a.i)), A::add(A::mul(c, a.i), A::mul(s, a.r))};
    } else {  // KPHASE, KT, KTDG: only bit-1 amplitudes change (callers skip bit 0)
        const T c = Coef<T>::c(g), s = Coef<T>::s(g);
        return Cx<T>{A::sub(A::mul(c, a.r), A::mul(s, a.i)), A::add(A::mul(c, a.i), A::mul(s, a.r))};
    }
}

// Swap update for gate kind K: the amplitude arriving from the partner (reference: x_core,
// y_core).
template <class T, uint32_t K>
__device__ __forceinline__ Cx<T> swap_update(bool bit, Cx<T> b) {
    if constexpr (K == KX) return b;
    else return bit ? Cx<T>{neg(b.i), b.r} : Cx<T>{b.i, neg(b.r)};   // Y
}

// Kind parameter of the update templates meaning "the kind is only known at run time".
constexpr uint32_t KANY = 0xFFu;

// Run-time dispatch of the updates (one copy of each kind's code per call site).
template <class T, class G>
__device__ __forceinline__ Cx<T> branch_update_rt(uint32_t kind, const G& g, bool bit, Cx<T> a, Cx<T> b) {
    switch (kind) {
    case KH: return branch_update<T, KH>(g, bit, a, b);
    case KRX: return branch_update<T, KRX>(g, bit, a, b);
    case KRY: return branch_update<T, KRY>(g, bit, a, b);
    default: return branch_update<T, KU>(g, bit, a, b);
    }
}

template <class T, class G>
__device__ __forceinline__ Cx<T> diag_update_rt(uint32_t kind, const G& g, bool bit, Cx<T> a) {
    switch (kind) {
    case KZ: return diag_update<T, KZ>(g, bit, a);
    case KS: return diag_update<T, KS>(g, bit, a);
    case KSDG: return diag_update<T, KSDG>(g, bit, a);
    case KYPH: return diag_update<T, KYPH>(g, bit, a);
    case KRZ: return diag_update<T, KRZ>(g, bit, a);
    default: return diag_update<T, KPHASE>(g, bit, a);
    }
}

template <class T>
__device__ __forceinline__ Cx<T> swap_update_rt(uint32_t kind, bool bit, Cx<T> b) {
    return kind == KX ? swap_update<T, KX>(bit, b) : swap_update<T, KY>(bit, b);
}

__host__ __device__ constexpr bool branch_kind(uint32_t k) { return k == KH || k == KRX || k == KRY || k == KU; }
__host__ __device__ constexpr bool swap_kind(uint32_t k) { return k == KX || k == KY; }
__host__ __device__ constexpr bool one_sided_kind(uint32_t k) {
    return k == KZ || k == KS || k == KSDG || k == KPHASE || k == KT || k == KTDG;
}

// Prune rule of the reference (emulator/include/data_t.h:50-60): |re| < thr && |im| < thr,
// decided in FP64. For doubles |x| < thr is compared on the bit patterns (non-negative
// doubles order like their bits; NaN compares false as in the FP64 test). For floats the
// host passes the largest float f with (double)f < thr, so |x| <= f is the same FP64 test.
__device__ __forceinline__ bool negligible(Cx<double> v, const PruneBits& t) {
    const unsigned long long m = 0x7FFFFFFFFFFFFFFFULL;
    return ((unsigned long long)__double_as_longlong(v.r) & m) < t.d &&
           ((unsigned long long)__double_as_longlong(v.i) & m) < t.d;
}
// FP32 compares issue on the wide FP32 pipes and take |x| as an operand modifier: one compare
// per component (NaN compares false, as its bit pattern does above t.f).
__device__ __forceinline__ bool negligible(Cx<float> v, const PruneBits& t) {
    const float f = __int_as_float((int)t.f);
    return fabsf(v.r) <= f && fabsf(v.i) <= f;
}

// ---- asynchronous global -> shared copies (sm_80+ PTX) ----------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Asynchronous 16-byte global -> shared copy (both addresses 16-byte aligned), L2 only.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Close the thread's current group of cp.async copies.
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Wait until at most N of the thread's committed cp.async groups are still in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

}  // namespace sqc
