// zc_push_exact.cu -- the exact build of the push + deposit kernels
// (zc_push_impl.cuh).  Compiled with --fmad=false: every float32 operation rounds as
// in the reference C.
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace exact {
#include "zc_push_impl.cuh"
}  // namespace exact

cudaError_t launch_push_tiles_exact(const PushLaunch &a, cudaStream_t st) {
  return exact::launch_push_tiles_variant(a, st);
}

cudaError_t launch_push_spill_exact(const float *EB, float *J, const Grid &G, const Particles &sin, const int *sin_cnt,
                                 int sin_cap, const Spill &S, double *ekin, int *err, const PushConst &C,
                                 int nblocks, cudaStream_t st) {
  return exact::launch_push_spill_variant(EB, J, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks, st);
}

}  // namespace zc
