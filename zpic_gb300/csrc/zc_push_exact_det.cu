// zc_push_exact_det.cu -- the exact build of the push + deposit kernels in
// deterministic mode (zc_push_impl.cuh with DET = true: currents and
// kinetic energy accumulated as 64-bit fixed point).  Compiled with
// --fmad=false, as zc_push_exact.cu.
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace exact_det {
#include "zc_push_impl.cuh"
}  // namespace exact_det

cudaError_t prepare_push_tiles_exact_det(int TX, int TY) { return exact_det::prepare_push_variant<true>(TX, TY); }

cudaError_t launch_push_tiles_exact_det(const PushLaunch &a, cudaStream_t st) {
  return exact_det::launch_push_tiles_variant<true>(a, st);
}

ZC_SPILL_LAUNCHER(launch_push_spill_exact_det) {
  return exact_det::launch_push_spill_variant<true>(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks,
                                                    st);
}

}  // namespace zc
