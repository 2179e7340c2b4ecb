// zc_push_fast_det.cu -- the fast build of the push + deposit kernels in
// deterministic mode (zc_push_impl.cuh with DET = true: currents and
// kinetic energy accumulated as 64-bit fixed point).  Compiled with the
// flags of zc_push_fast.cu.
#define ZC_FAST_ALGEBRA 1  // re-associated current weights (zc_push_impl.cuh)
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace fast_det {
#include "zc_push_impl.cuh"
}  // namespace fast_det

cudaError_t prepare_push_tiles_fast_det(int TX, int TY) { return fast_det::prepare_push_variant<true>(TX, TY); }

cudaError_t launch_push_tiles_fast_det(const PushLaunch &a, cudaStream_t st) {
  return fast_det::launch_push_tiles_variant<true>(a, st);
}

ZC_SPILL_LAUNCHER(launch_push_spill_fast_det) {
  return fast_det::launch_push_spill_variant<true>(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks,
                                                   st);
}

}  // namespace zc
