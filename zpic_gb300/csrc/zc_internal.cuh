// zc_internal.cuh -- device-side layout and helpers shared by the kernels of
// libzpic_cuda (GB300, sm_103a).
//
// Grid layout in HBM (one allocation per field set):
//   planes [component][row][column], `pitch` floats per row (a multiple of 32,
//   so every row starts on a 128-byte boundary and TMA boxes can start on any
//   multiple of 4 columns), `rows` = ny + 3 rows.
//   Buffer coordinates: column i+1, row j+1 hold cell (i, j); columns/rows
//   0, nx+1, nx+2 (resp. ny) are the guard cells of the reference layout
//   (1 lower, 2 upper; em2d/emf.c:59-89).
//   E and B share one 6-plane allocation (Ex Ey Ez Bx By Bz) so the particle
//   kernel stages both with a single 3-D TMA box.
//
// Particle layout (one species): two arrays of 16- and 8-byte records,
//   u[k]  = (ux, uy, uz, cell)   float32 proper velocity; the cell indices
//           ix | iy << 16 stored in the bits of the fourth word
//   xy[k] = (x, y)               float32 in-cell position in [0, 1]
// -- the same quantities as t_part (em2d/particles.h:29-37), 24 bytes per
// particle moved with two vector accesses -- partitioned into rectangular
// tiles of TX x TY cells.  Tile t owns the contiguous segment
// [off[t], off[t] + cap[t]); its first np[t] slots are in use.  Two copies
// (A, B) alternate every step.
//
// Slots keep their particle from step to step: the push writes a particle
// back to the slot it came from, and a particle that leaves the tile leaves
// a hole there (cell word kHole); particles arriving from other tiles are
// appended after slot np.  The periodic cell sort compacts the holes away
// and stores the tile in cell order, every full chunk of 32 * kLaneRun
// particles transposed (tile_slot: particle l * kLaneRun + k of the chunk
// at slot k * 32 + l).  A push warp reads and writes slot k * 32 + l at its
// k-th step (coalesced), so lane l meets the chunk's particles
// l * kLaneRun ... l * kLaneRun + kLaneRun - 1 one after another, which lie
// in one or two cells.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace zc {

// error bits accumulated on the device and read back by the host
enum : int {
  ERR_TIMEOUT = 1,       // a bounded TMA barrier wait gave up
  ERR_ESCAPE = 2,        // particle outside its cell/tile (moved > 1 cell)
  ERR_OVERFLOW = 4,      // spill buffer full: particles lost
  ERR_SPILLED = 8,       // particles went to the spill buffer (host re-layout due)
};

struct Particles {       // one particle buffer
  float4 *u;             // ux, uy, uz, packed cell
  float2 *xy;            // x, y
};

// particles a push lane takes from one chunk, one after another
#ifndef ZC_LANE_RUN
#define ZC_LANE_RUN 8
#endif
constexpr int kLaneRun = ZC_LANE_RUN;
constexpr int kChunk = 32 * kLaneRun;
// cell word of an empty slot (no cell has both indices 0xffff: grids have at
// most 65535 cells per axis)
constexpr unsigned kHole = 0xffffffffu;

struct PRec {            // one particle in registers
  int ix, iy;
  float x, y, ux, uy, uz;
};

#ifdef __CUDACC__
__device__ __forceinline__ PRec load_particle(const Particles &p, long long k) {
  const float4 u = p.u[k];
  const float2 r = p.xy[k];
  const unsigned c = (unsigned)__float_as_int(u.w);
  PRec q;
  q.ix = (int)(c & 0xffffu);
  q.iy = (int)(c >> 16);
  q.x = r.x;
  q.y = r.y;
  q.ux = u.x;
  q.uy = u.y;
  q.uz = u.z;
  return q;
}

__device__ __forceinline__ void load_cell(const Particles &p, long long k, int &ix, int &iy) {
  const unsigned c = (unsigned)__float_as_int(p.u[k].w);
  ix = (int)(c & 0xffffu);
  iy = (int)(c >> 16);
}

// cells are in [0, 65535] (grids are limited to 65535 cells per axis)
__device__ __forceinline__ void store_particle(const Particles &p, long long k, int ix, int iy, float x, float y,
                                               float ux, float uy, float uz) {
  p.u[k] = make_float4(ux, uy, uz, __int_as_float((int)((unsigned)ix | ((unsigned)iy << 16))));
  p.xy[k] = make_float2(x, y);
}

__device__ __forceinline__ void store_particle(const Particles &p, long long k, const PRec &q) {
  store_particle(p, k, q.ix, q.iy, q.x, q.y, q.ux, q.uy, q.uz);
}

__device__ __forceinline__ bool is_hole_word(float w) { return (unsigned)__float_as_int(w) == kHole; }
__device__ __forceinline__ bool is_hole(const Particles &p, long long k) { return is_hole_word(p.u[k].w); }
__device__ __forceinline__ void store_hole(const Particles &p, long long k) {
  p.u[k] = make_float4(0.f, 0.f, 0.f, __int_as_float((int)kHole));
}
#endif

// Slot of the i-th particle (in cell order) of a tile of n particles in the
// lane-run layout: full chunks of kChunk particles transposed (particle
// l * kLaneRun + k of a chunk at slot k * 32 + l), the last, partial chunk
// in order.
__host__ __device__ __forceinline__ int tile_slot(int i, int n) {
  const int c0 = i & ~(kChunk - 1);
  if (c0 + kChunk > n) return i;
  const int r = i - c0;
  return c0 + (r % kLaneRun) * 32 + r / kLaneRun;
}

struct Grid {            // geometry of the padded SoA grids
  int nx, ny;            // interior cells
  int pitch, rows;       // floats per row, rows per plane
  size_t plane;          // floats per plane (pitch * rows)
};

// bounded spin limit for mbarrier waits: each try_wait can suspend for a
// while, so this is many milliseconds at least
constexpr int kWaitIters = 1 << 20;

// ---------------------------------------------------------------------------
// PTX wrappers: mbarrier + TMA (cp.async.bulk.tensor) for sm_90+ / sm_103a
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; returns false when the limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < kWaitIters; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// element-wise atomic add of a shared-memory box into global memory
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap *map, const void *src, int x, int y,
                                                  int z) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%2, %3, %4}], [%1];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group"
      " [%0, {%2, %3, %4}], [%1];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// Ampere-style per-thread asynchronous copies global -> shared (16 or 8
// bytes, naturally aligned)
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// 4-byte copy; with `valid` false the destination is zero-filled and nothing
// is read from `src` (which must still be a mapped address)
__device__ __forceinline__ void cp_async4_zfill(void *dst, const void *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// contiguous bulk copy global -> shared, completing on an mbarrier (both
// addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---------------------------------------------------------------------------
// block-wide exclusive scan of one int per thread (NT threads, NT % 32 == 0);
// `swarp` holds NT/32 ints of shared memory; all threads must call it.
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ int block_exclusive_scan(int v, int &total, int *swarp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) swarp[warp] = x;
  __syncthreads();
  int before = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < NT / 32; ++w) {
    int c = swarp[w];
    before += (w < warp) ? c : 0;
    tot += c;
  }
  __syncthreads();
  total = tot;
  return before + x - v;
}

// block-wide sum of a double, result valid in thread 0; `sred` NT/32 doubles
template <int NT>
__device__ __forceinline__ double block_sum_double(double v, double *sred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sred[warp] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += sred[w];
  }
  __syncthreads();
  return s;
}

}  // namespace zc
