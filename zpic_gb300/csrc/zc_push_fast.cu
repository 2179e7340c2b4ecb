// zc_push_fast.cu -- the fast build of the push + deposit kernels
// (zc_push_impl.cuh).  Compiled with FMA contraction and approximate float32 division / square
// root: same algorithm, results within a few float32 ulps per operation of
// the exact build.  The deterministic-mode variants are in zc_push_fast_det.cu.
#define ZC_FAST_ALGEBRA 1  // re-associated current weights (zc_push_impl.cuh)
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace fast {
#include "zc_push_impl.cuh"
}  // namespace fast

cudaError_t launch_push_tiles_fast(const PushLaunch &a, cudaStream_t st) {
  return fast::launch_push_tiles_variant<false>(a, st);
}

ZC_SPILL_LAUNCHER(launch_push_spill_fast) {
  return fast::launch_push_spill_variant<false>(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks, st);
}

}  // namespace zc
