// Host-side launchers of the engine's kernels. Every launcher enqueues on the given stream
// and returns the launch status; none synchronizes.
#pragma once
#include <cuda_runtime_api.h>
#include "sqc_types.h"
#ifdef __CUDACC__
#include "sqc_device.cuh"
#endif

namespace sqc {

cudaError_t launch_pass(const PassArgs& a, bool dbl, int sms, cudaStream_t st);
cudaError_t launch_set_zero(const TableDev& t, Ctl* ctl, int p, bool dbl, cudaStream_t st);
cudaError_t launch_set_state(const unsigned long long* keys, const double* re, const double* im,
                             unsigned long long n, const TableDev& t, Ctl* ctl, int p, bool dbl, int sms,
                             cudaStream_t st);
cudaError_t launch_count(const TableDev& t, Ctl* ctl, int p, int sms, cudaStream_t st);
cudaError_t launch_readout(const TableDev& t, Ctl* ctl, int p, bool dbl, unsigned long long* okeys, double* ore,
                           double* oim, unsigned long long cap, bool drop_negl, PruneBits pb, int sms,
                           cudaStream_t st);
cudaError_t launch_norm(const TableDev& t, Ctl* ctl, int p, bool dbl, int sms, cudaStream_t st);
cudaError_t launch_compare(const TableDev& ta, unsigned ep_a, bool dbl_a, const TableDev& tb, unsigned ep_b,
                           bool dbl_b, Ctl* out, int sms, cudaStream_t st);
cudaError_t launch_rehash(const TableDev& told, unsigned ep_old, const TableDev& tnew, unsigned ep_new,
                          int amp_bytes, Ctl* ctl, int sms, cudaStream_t st);

}  // namespace sqc
