// Host-side launchers of the engine's kernels. Every launcher enqueues on the given stream
// and returns the launch status; none synchronizes. list_hint is an upper bound on the
// state's live-bucket count, used only to size grids (the kernels read the exact count).
#pragma once
#include <cuda_runtime_api.h>
#include "sqc_types.h"
#ifdef __CUDACC__
#include "sqc_device.cuh"
#endif

namespace sqc {

// One gate pass (sqc_pass.cu): the direct kernel (tables up to 2^20 buckets), or the resolve
// kernel (pair and quad passes) and the staged kernel. Returns the number of kernels launched,
// or -1 when a launch failed.
int launch_pass(const PassArgs& a, unsigned long long list_hint, bool dbl, int sms, cudaStream_t st);
// Tables small enough for tiny_kernel: every pass of a flush in one single-block launch.
bool tiny_table(unsigned long long buckets);
// The passes (device array of np records; a's per-pass fields are ignored) in one launch.
int launch_tiny(const PassArgs& a, const TinyPass* passes, uint32_t np, bool dbl, cudaStream_t st);
cudaError_t launch_set_zero(const TableDev& t, Ctl* ctl, bool dbl, cudaStream_t st);
cudaError_t launch_set_state(const unsigned long long* keys, const double* re, const double* im,
                             unsigned long long n, const TableDev& t, Ctl* ctl, bool dbl, int sms,
                             cudaStream_t st);
cudaError_t launch_count(const TableDev& t, Ctl* ctl, unsigned long long list_hint, int sms, cudaStream_t st);
// Readout of the present entries whose stored key k has (k & smask) == sval (all by default).
cudaError_t launch_readout(const TableDev& t, Ctl* ctl, unsigned long long list_hint, unsigned long long frame,
                           bool dbl, unsigned long long* okeys, double* ore, double* oim, unsigned long long cap,
                           bool drop_negl, PruneBits pb, int sms, cudaStream_t st, unsigned long long smask = 0,
                           unsigned long long sval = 0);
// Exact sum of |a|^2 into sums->c[SUM_NORM] (sqc_exact.cuh); the caller zeroes it first.
cudaError_t launch_norm(const TableDev& t, Ctl* ctl, unsigned long long list_hint, bool dbl, ExactSums* sums, int sms,
                        cudaStream_t st);
cudaError_t launch_compare(const TableDev& ta, const Ctl* ca, unsigned long long hint_a, bool dbl_a,
                           const TableDev& tb, const Ctl* cb, unsigned long long hint_b, bool dbl_b,
                           unsigned long long d, Ctl* out, ExactSums* sums, int sms, cudaStream_t st);
// Measured FP64 fused multiply-add rate of the current device (lane operations per second), from
// a timed loop of independent FMA chains over sms * 8 blocks. Synchronizes the device.
cudaError_t measure_fp64_rate(int sms, double* fma_per_s);
cudaError_t launch_rehash(const TableDev& told, unsigned long long n_old, const TableDev& tnew, unsigned ep_new,
                          int amp_bytes, Ctl* ctl, int sms, cudaStream_t st);

}  // namespace sqc
