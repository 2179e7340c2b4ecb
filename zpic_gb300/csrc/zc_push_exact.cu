// zc_push_exact.cu -- the exact build of the push + deposit kernels
// (zc_push_impl.cuh).  Compiled with --fmad=false: every float32 operation rounds as in
// the reference C.  The deterministic-mode variants are in zc_push_exact_det.cu.
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {
namespace exact {
#include "zc_push_impl.cuh"
}  // namespace exact

cudaError_t launch_push_tiles_exact(const PushLaunch &a, cudaStream_t st) {
  return exact::launch_push_tiles_variant<false>(a, st);
}

ZC_SPILL_LAUNCHER(launch_push_spill_exact) {
  return exact::launch_push_spill_variant<false>(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks, st);
}

}  // namespace zc
