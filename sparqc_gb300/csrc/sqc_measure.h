// Launchers of the readout and measurement kernels (sqc_measure.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime_api.h>

#include "sqc_types.h"

namespace sqc {

// Device arrays of a key sort: entries (keys_in, re_in, im_in) of a readout are reordered by
// key into (keys_out, re_out, im_out); cum receives the inclusive cumulative |a|^2 when asked.
struct SortBuffers {
    unsigned long long* keys_in = nullptr;
    double* re_in = nullptr;
    double* im_in = nullptr;
    unsigned long long* keys_out = nullptr;
    double* re_out = nullptr;
    double* im_out = nullptr;
    unsigned* idx_in = nullptr;
    unsigned* idx_out = nullptr;
    double* cum = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
};

// sums->c[SUM_NORM] += sum of |a|^2 over present stored keys with (key & smask) == sval
// (exact; the caller zeroes it first).
cudaError_t launch_pattern_prob(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl,
                                unsigned long long smask, unsigned long long sval, ExactSums* sums, int sms,
                                cudaStream_t st);
// Remove present keys with (key & smask) != sval, scale the others by `scale`, set nnz.
cudaError_t launch_collapse(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl,
                            unsigned long long smask, unsigned long long sval, double scale, int sms, cudaStream_t st);
// Scratch bytes for sorting (and scanning) n entries.
size_t sort_scratch_bytes(unsigned long long n);
// Sort n readout entries by their low key_bits bits; with_cum also fills sb.cum.
cudaError_t sort_entries(SortBuffers& sb, unsigned long long n, uint32_t key_bits, bool with_cum, int sms,
                         cudaStream_t st);
// shots samples from key-sorted entries with inclusive cumulative probabilities cum.
cudaError_t launch_sample(const unsigned long long* keys, const double* cum, unsigned long long n,
                          unsigned long long seed, unsigned long long shots, unsigned long long* out, int sms,
                          cudaStream_t st);

}  // namespace sqc
