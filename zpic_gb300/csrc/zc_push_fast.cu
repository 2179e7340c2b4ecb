// zc_push_fast.cu -- the fast build of the push + deposit kernels
// (zc_push_impl.cuh).  Compiled with FMA contraction and approximate float32 division / square
// root: same algorithm, results within a few float32 ulps per operation of
// the exact build.
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace fast {
#include "zc_push_impl.cuh"
}  // namespace fast

cudaError_t launch_push_tiles_fast(const PushLaunch &a, cudaStream_t st) {
  return fast::launch_push_tiles_variant(a, st);
}

cudaError_t launch_push_spill_fast(const float *EB, float *J, const Grid &G, const Particles &sin, const int *sin_cnt,
                                 int sin_cap, const Spill &S, double *ekin, int *err, const PushConst &C,
                                 int nblocks, cudaStream_t st) {
  return fast::launch_push_spill_variant(EB, J, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks, st);
}

}  // namespace zc
