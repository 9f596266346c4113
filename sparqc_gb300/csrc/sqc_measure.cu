// Readout and measurement on the device: pattern probabilities, projective measurement of a
// qubit with collapse, key-sorted readout and sampling.
//
// The reference reads the whole dense buffer back and filters and orders it on the host
// (emulator/device/table.cuh:47-75, Circuit__::get_state_full, emulator/include/circuit.h:
// 206-253, whose state_to_choose pattern is the (mask, value) pair here). Here the filter,
// the key sort and the probability sums run on the GPU and only the selected entries travel.
//
// Keys in the table are stored in the planner's frame (stored = actual ^ frame); a pattern on
// actual keys (actual & mask) == value is tested as (stored & mask) == (value ^ (frame & mask)).
// Probability sums are exact (sqc_exact.cuh) and rounded once, so they do not depend on the
// order in which the warps meet the keys; a measurement outcome is reproducible.
#include <algorithm>

#include <cub/cub.cuh>

#include "sqc_exact.cuh"
#include "sqc_kernels.h"
#include "sqc_measure.h"

namespace sqc {
namespace {

template <class T>
__device__ __forceinline__ Cx<T> amp_at(const void* amps, size_t s) {
    if constexpr (sizeof(T) == 8) {
        const double2 v = reinterpret_cast<const double2*>(amps)[s];
        return Cx<T>{v.x, v.y};
    } else {
        const float2 v = reinterpret_cast<const float2*>(amps)[s];
        return Cx<T>{v.x, v.y};
    }
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// sums->c[SUM_NORM] += sum of |a|^2 over present keys with (stored & smask) == sval, exactly.
template <class T>
__global__ void pattern_prob_kernel(TableDev t, Ctl* ctl, unsigned long long smask, unsigned long long sval,
                                    ExactSums* sums) {
    const unsigned long long n = ctl->list_n;
    unsigned long long acc[kSumChunks] = {};
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const size_t slot = (size_t)t.list[s >> kSlotBits] * kSlots + (s & 15);
        const unsigned long long key = t.keys[slot];
        if (!((int)(key & 15ULL) == (int)(s & 15)) || (key & smask) != sval) continue;
        const Cx<T> v = amp_at<T>(t.amps, slot);
        const double r = (double)v.r, i = (double)v.i;
        exact_add_prod(acc, r, r);
        exact_add_prod(acc, i, i);
    }
    exact_flush(acc, sums->c[SUM_NORM]);
}

// Projective collapse: present keys with (stored & smask) != sval are removed, the others
// scaled by `scale`; the kept count goes to out_count.
template <class T>
__global__ void collapse_kernel(TableDev t, Ctl* ctl, unsigned long long smask, unsigned long long sval, double scale) {
    const unsigned long long n = ctl->list_n;
    unsigned long long kept = 0;
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < n * kSlots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const int j = (int)(s & 15);
        const size_t slot = (size_t)t.list[s >> kSlotBits] * kSlots + j;
        const unsigned long long key = t.keys[slot];
        if ((int)(key & 15ULL) != j) continue;
        if ((key & smask) != sval) {
            t.keys[slot] = empty_key(j);
            continue;
        }
        ++kept;
        if constexpr (sizeof(T) == 8) {
            double2* a = reinterpret_cast<double2*>(t.amps) + slot;
            const double2 v = *a;
            *a = make_double2(__dmul_rn(v.x, scale), __dmul_rn(v.y, scale));
        } else {
            float2* a = reinterpret_cast<float2*>(t.amps) + slot;
            const float2 v = *a;
            const float f = (float)scale;
            *a = make_float2(__fmul_rn(v.x, f), __fmul_rn(v.y, f));
        }
    }
    for (int o = 16; o; o >>= 1) kept += __shfl_down_sync(kFull, kept, o);
    if ((threadIdx.x & 31) == 0 && kept) atomicAdd(&ctl->out_count, kept);
}

__global__ void set_nnz_kernel(Ctl* ctl) { ctl->nnz = ctl->out_count; }

__global__ void iota_kernel(unsigned* idx, unsigned long long n) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        idx[i] = (unsigned)i;
}

// Gather amplitudes in sorted order and, when cum is given, |a|^2 per entry.
__global__ void gather_kernel(const unsigned* idx, const double* re_in, const double* im_in, double* re_out,
                              double* im_out, double* prob, unsigned long long n) {
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned k = idx[i];
        const double r = re_in[k], im = im_in[k];
        re_out[i] = r;
        im_out[i] = im;
        if (prob) prob[i] = __fma_rn(r, r, __dmul_rn(im, im));
    }
}

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

// Shot s draws u = uniform(seed, s) * total and takes the first entry whose inclusive
// cumulative probability exceeds u.
__global__ void sample_kernel(const unsigned long long* keys, const double* cum, unsigned long long n,
                              unsigned long long seed, unsigned long long shots, unsigned long long* out) {
    if (n == 0) return;
    const double total = cum[n - 1];
    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < shots;
         s += (unsigned long long)gridDim.x * blockDim.x) {
        const double u = (double)(splitmix(seed ^ splitmix(s)) >> 11) * (1.0 / 9007199254740992.0) * total;
        unsigned long long lo = 0, hi = n - 1;
        while (lo < hi) {
            const unsigned long long mid = (lo + hi) >> 1;
            if (cum[mid] > u) hi = mid;
            else lo = mid + 1;
        }
        out[s] = keys[lo];
    }
}

int grid_of(unsigned long long items, int sms) {
    const unsigned long long g = (items + 255) / 256;
    return (int)std::max<unsigned long long>(1, std::min<unsigned long long>(g, (unsigned long long)sms * 8));
}

}  // namespace

cudaError_t launch_pattern_prob(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl,
                                unsigned long long smask, unsigned long long sval, ExactSums* sums, int sms,
                                cudaStream_t st) {
    const int g = grid_of(list_hint * kSlots + 1, sms);
    if (dbl) pattern_prob_kernel<double><<<g, 256, 0, st>>>(t, ctl, smask, sval, sums);
    else pattern_prob_kernel<float><<<g, 256, 0, st>>>(t, ctl, smask, sval, sums);
    return cudaGetLastError();
}

cudaError_t launch_collapse(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl,
                            unsigned long long smask, unsigned long long sval, double scale, int sms, cudaStream_t st) {
    const int g = grid_of(list_hint * kSlots + 1, sms);
    cudaMemsetAsync(&ctl->out_count, 0, sizeof(unsigned long long), st);
    if (dbl) collapse_kernel<double><<<g, 256, 0, st>>>(t, ctl, smask, sval, scale);
    else collapse_kernel<float><<<g, 256, 0, st>>>(t, ctl, smask, sval, scale);
    set_nnz_kernel<<<1, 1, 0, st>>>(ctl);
    return cudaGetLastError();
}

size_t sort_scratch_bytes(unsigned long long n) {
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (const unsigned*)nullptr, (unsigned*)nullptr, (int)n);
    cub::DeviceScan::InclusiveSum(nullptr, b, (const double*)nullptr, (double*)nullptr, (int)n);
    return std::max(a, b) + 256;
}

cudaError_t sort_entries(SortBuffers& sb, unsigned long long n, uint32_t key_bits, bool with_cum, int sms,
                         cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    iota_kernel<<<grid_of(n, sms), 256, 0, st>>>(sb.idx_in, n);
    size_t bytes = sb.tmp_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(sb.tmp, bytes, sb.keys_in, sb.keys_out, sb.idx_in, sb.idx_out,
                                                    (int)n, 0, (int)key_bits, st);
    if (e != cudaSuccess) return e;
    gather_kernel<<<grid_of(n, sms), 256, 0, st>>>(sb.idx_out, sb.re_in, sb.im_in, sb.re_out, sb.im_out,
                                                   with_cum ? sb.cum : nullptr, n);
    if (with_cum) {
        bytes = sb.tmp_bytes;
        e = cub::DeviceScan::InclusiveSum(sb.tmp, bytes, sb.cum, sb.cum, (int)n, st);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t launch_sample(const unsigned long long* keys, const double* cum, unsigned long long n,
                          unsigned long long seed, unsigned long long shots, unsigned long long* out, int sms,
                          cudaStream_t st) {
    sample_kernel<<<grid_of(shots, sms), 256, 0, st>>>(keys, cum, n, seed, shots, out);
    return cudaGetLastError();
}

}  // namespace sqc
