// zc_particles.cu -- particle bookkeeping kernels of libzpic_cuda (sm_103a):
// tile migration, per-tile cell sort, re-layout (upload, injection, capacity
// changes), download, charge density and the kinetic-energy sum.  The push
// and deposit kernels themselves live in zc_push_impl.cuh (compiled twice,
// exact and fast, by zc_push_exact.cu / zc_push_fast.cu).
//
//   k_migrate     one CTA per tile: appends the particles bound for it that
//                 wait in the outboxes of its (up to 8) neighbours (the push
//                 does this itself; this kernel settles the outboxes before
//                 the particles are read back, counted or re-laid out).
//   k_cellsort    one CTA per tile: counting sort of the tile by cell (holes
//                 dropped), so that the push lanes meet runs of one cell.
//   re-layout     upload, moving-window injection and capacity changes.
#include <algorithm>
#include <atomic>

#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {

// ---------------------------------------------------------------------------
// K2: migrate the outboxes into the destination tiles, one CTA per tile
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT) k_migrate(Particles pout, TileSet T, Outbox O, Spill S, int *err,
                                                int ntx, int nty, int mw) {
  __shared__ int swarp[NT / 32];
  __shared__ int nb[8];
  __shared__ int nnb;
  const int t = blockIdx.x;
  const int tx = t % ntx, ty = t / ntx;
  if (threadIdx.x == 0) {
    int c = 0;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy) continue;
        int x = tx + dx, y = ty + dy;
        y += (y < 0) ? nty : 0;
        y -= (y >= nty) ? nty : 0;
        if (x < 0 || x >= ntx) {
          if (mw) continue;
          x = (x + ntx) % ntx;
        }
        const int id = x + y * ntx;
        bool dup = (id == t);
        for (int m = 0; m < c; ++m) dup |= (nb[m] == id);
        if (!dup) nb[c++] = id;
      }
    nnb = c;
  }
  __syncthreads();
  int errbits = 0;
  const int stay = T.np[t];
  const long long start = (long long)T.off[t] + stay;
  const int room = T.cap[t] - stay;
  int placed = 0;
  for (int m = 0; m < nnb; ++m) {
    const int src = nb[m];
    const int n = O.cnt[src];
    const long long ob = (long long)src * O.cap;
    for (int e0 = 0; e0 < n; e0 += NT) {
      const int e = e0 + threadIdx.x;
      const int f = (e < n && O.dst[ob + e] == t) ? 1 : 0;
      int tot;
      const int pre = block_exclusive_scan<NT>(f, tot, swarp);
      if (f) {
        const long long q = ob + e;
        const int s = placed + pre;
        if (s < room)
          store_particle(pout, start + s, load_particle(O.p, q));
        else
          spill_particle(S, &errbits, load_particle(O.p, q));
      }
      placed += tot;
    }
  }
  if (threadIdx.x == 0) T.np[t] = stay + min(placed, room);
  if (errbits) atomicOr(err, errbits);
}

// ---------------------------------------------------------------------------
// re-layout: counting, scattering, per-tile ordering
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tile_of(int ix, int iy, const LayoutConst &L) {
  return (ix / L.TX) + (iy / L.TY) * L.ntx;
}

// adds n_lanes to counter[t] for every group of the calling (active) lanes
// that share t, with one atomic per group; returns the counter's old value
// plus this lane's rank in its group (lists in cell order put most lanes of
// a warp on one tile)
__device__ __forceinline__ int warp_grouped_add(int *counter, int t) {
  const unsigned am = __activemask();
  const unsigned same = __match_any_sync(am, t);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(same) - 1;
  int first = 0;
  if (lane == leader) first = atomicAdd(&counter[t], __popc(same));
  first = __shfl_sync(same, first, leader);
  return first + __popc(same & ((1u << lane) - 1));
}

// AoS records (7 words: ix, iy, x, y, ux, uy, uz) -> SoA list.  A CTA of
// 256 threads reads its 256 records as 1792 consecutive words into shared
// memory (coalesced whether the records sit in device memory or in mapped
// host memory, read straight over the host link), then every thread takes
// one record (stride 7 words: no bank conflicts).  cell_cnt (nx * ny
// counters), when given, receives the particles of every cell.
__global__ void __launch_bounds__(256) k_stage_to_list(const int *w, int n, Particles list, int *cell_cnt,
                                                       LayoutConst L, int *err) {
  __shared__ int sw[256 * 7];
  for (long long b0 = (long long)blockIdx.x * 256; b0 < n; b0 += (long long)gridDim.x * 256) {
    const int m = (int)min(256LL, n - b0);
    __syncthreads();
    for (int j = threadIdx.x; j < m * 7; j += 256) sw[j] = w[b0 * 7 + j];
    __syncthreads();
    if (threadIdx.x < m) {
      const int *r = sw + threadIdx.x * 7;
      int ix = r[0], iy = r[1];
      if (ix < 0 || ix >= L.nx || iy < 0 || iy >= L.ny) {
        atomicOr(err, ERR_ESCAPE);
        ix = min(max(ix, 0), L.nx - 1);
        iy = min(max(iy, 0), L.ny - 1);
      }
      store_particle(list, b0 + threadIdx.x, ix, iy, __int_as_float(r[2]), __int_as_float(r[3]),
                     __int_as_float(r[4]), __int_as_float(r[5]), __int_as_float(r[6]));
      if (cell_cnt) warp_grouped_add(cell_cnt, ix + iy * L.nx);
    }
  }
}

// Per tile (one CTA of 1024 threads, one thread per cell of the tile): the
// exclusive scan of its cell counts in the tile's cell order (local x
// fastest, as k_cellsort orders), written back in place as every cell's first
// position, and the tile's count into cnt.
__global__ void __launch_bounds__(1024) k_cell_starts(int *cell, int *cnt, LayoutConst L) {
  __shared__ int swarp[32];
  const int t = blockIdx.x;
  const int cx0 = (t % L.ntx) * L.TX, cy0 = (t / L.ntx) * L.TY;
  const int lx = threadIdx.x % L.TX, ly = threadIdx.x / L.TX;
  const int ix = cx0 + lx, iy = cy0 + ly;
  const bool in = threadIdx.x < L.TX * L.TY && ix < L.nx && iy < L.ny;
  const long long g = (long long)iy * L.nx + ix;
  const int v = in ? cell[g] : 0;
  int tot;
  const int pre = block_exclusive_scan<1024>(v, tot, swarp);
  if (in) cell[g] = pre;
  if (threadIdx.x == 0) cnt[t] = tot;
}

// list particles straight into the sorted tile layout: the particle takes the
// next position of its cell (cell starts from k_cell_starts) and is stored
// at that position's tile_slot, as k_cellsort places it
__global__ void k_scatter_sorted(Particles list, int n, Particles dst, const int *off, const int *cnt,
                                 int *cell_pos, LayoutConst L) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const PRec r = load_particle(list, k);
    const int t = tile_of(r.ix, r.iy, L);
    const int pos = warp_grouped_add(cell_pos, r.ix + r.iy * L.nx);
    store_particle(dst, (long long)off[t] + tile_slot(pos, cnt[t]), r);
  }
}

// counts the particles of a list per tile (list length read on the device)
__global__ void k_count_list(Particles list, const int *n_ptr, int n_cap, int *cnt, LayoutConst L) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
  {
    int ix, iy;
    load_cell(list, k, ix, iy);
    warp_grouped_add(cnt, tile_of(ix, iy, L));
  }
}

// tile particles keep their tile: copy to the new offsets, holes dropped
// (one CTA of 256 threads per tile)
__global__ void __launch_bounds__(256) k_copy_tiles(Particles src, const int *off_old, const int *np_old,
                                                    Particles dst, const int *off_new, int *fill) {
  __shared__ int swarp[8];
  const int t = blockIdx.x;
  const int n = np_old[t];
  const long long a = off_old[t], b = off_new[t];
  int placed = 0;
  for (int k0 = 0; k0 < n; k0 += 256) {
    const int k = k0 + threadIdx.x;
    const bool f = k < n && !is_hole(src, a + k);
    int tot;
    const int pre = block_exclusive_scan<256>(f ? 1 : 0, tot, swarp);
    if (f) {
      const int q = placed + pre;
      store_particle(dst, b + q, load_particle(src, a + k));
    }
    placed += tot;
  }
  if (threadIdx.x == 0) fill[t] = placed;
}

// particles (not holes) in every tile's slots
__global__ void __launch_bounds__(256) k_count_valid(Particles buf, const int *off, const int *np, int *cnt) {
  __shared__ int swarp[8];
  const int t = blockIdx.x;
  const int n = np[t];
  const long long a = off[t];
  int c = 0;
  for (int k = threadIdx.x; k < n; k += 256) c += is_hole(buf, a + k) ? 0 : 1;
  int tot;
  block_exclusive_scan<256>(c, tot, swarp);
  if (threadIdx.x == 0) cnt[t] = tot;
}

// list particles are appended to their tile
__global__ void k_scatter_list(Particles list, const int *n_ptr, int n_cap, Particles dst, const int *off,
                               const int *cap, int *fill, LayoutConst L, int *err) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const PRec r = load_particle(list, k);
    const int t = tile_of(r.ix, r.iy, L);
    const int s = warp_grouped_add(fill, t);
    if (s < cap[t]) {
      const long long q = (long long)off[t] + s;
      store_particle(dst, q, r);
    } else {
      atomicOr(err, ERR_OVERFLOW);  // capacities are sized from exact counts: cannot happen
    }
  }
}

// Counting sort of every tile by local cell (one CTA of 1024 threads per
// tile, src -> dst at the same offsets): a shared-memory histogram, a scan,
// then every particle takes the next position of its cell, stored at its
// tile_slot (the lane-run layout); holes are dropped and np becomes the
// particle count.  The order inside a cell follows the atomics' timing.  The
// reference sorts its whole buffer by cell every n_sort steps for cache
// reuse (spec_sort, em2d/particles.c:942-1007); here the per-tile sort gives
// the push lanes runs of particles in one cell.
//
// The tile is staged in shared memory by bulk copies (TMA) of its records,
// 16 + 8 bytes a particle, that one thread starts: a whole tile is in flight
// at once, without a load instruction a particle; the count reads shared
// memory.  Tile offsets are multiples of 32 particles, so both copies start
// 16-byte aligned; an odd last float2 is loaded plainly.  The wait on the
// copies is bounded: on a timeout the tile is left as it was and the error
// word says so.  A tile that fits
// (n <= S) is then written out in slot order: every particle notes its index
// at its slot (a 16-bit permutation), and the threads store slot j = thread,
// thread + NT, ... from the staged records, coalesced (the lane-run layout
// would otherwise scatter every warp's stores over the tile).  A fuller tile
// stages its first S particles, reads the rest from global memory and
// scatters.  Dynamic shared memory: the cell cursors, then S float4, S float2
// and S 16-bit slots.
#ifndef ZC_SORT_NT
#define ZC_SORT_NT 1024
#endif
template <int NT>
__global__ void __launch_bounds__(NT, 2048 / NT) k_cellsort(Particles src, Particles dst, const int *off, int *np,
                                                             LayoutConst L, int S, int *err) {
  constexpr int MAXC = 1024, CPT = MAXC / NT;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  int *cursor = reinterpret_cast<int *>(sm_raw);
  float4 *su = reinterpret_cast<float4 *>(sm_raw + MAXC * sizeof(int));
  float2 *sxy = reinterpret_cast<float2 *>(su + S);
  unsigned short *perm = reinterpret_cast<unsigned short *>(sxy + S);
  __shared__ int swarp[NT / 32];
  __shared__ __align__(8) uint64_t bar;
  const int t = blockIdx.x;
  const int ncell = L.TX * L.TY;
  const int cx0 = (t % L.ntx) * L.TX, cy0 = (t / L.ntx) * L.TY;
  const int n = np[t];
  const int ns = min(n, S);
  const int nb = ns & ~1;  // float2 records copied in bulk (whole 16-byte units)
  const long long b = off[t];
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && ns > 0) {
    mbar_expect_tx(&bar, (uint32_t)ns * 16u + (uint32_t)nb * 8u);
    constexpr int kPiece = 4096;  // records a copy
    for (int k = 0; k < ns; k += kPiece)
      bulk_load(&su[k], &src.u[b + k], (uint32_t)min(kPiece, ns - k) * 16u, &bar);
    for (int k = 0; k < nb; k += kPiece)
      bulk_load(&sxy[k], &src.xy[b + k], (uint32_t)min(kPiece, nb - k) * 8u, &bar);
  }
  if (threadIdx.x == 0 && nb < ns) sxy[nb] = src.xy[b + nb];
  for (int c = threadIdx.x; c < MAXC; c += NT) cursor[c] = 0;
  auto cell_of_word = [&](float w) {  // -1 for a hole
    const unsigned u = (unsigned)__float_as_int(w);
    if (u == kHole) return -1;
    const int c = ((int)(u & 0xffffu) - cx0) + ((int)(u >> 16) - cy0) * L.TX;
    return min(max(c, 0), ncell - 1);
  };
  const bool loaded = ns == 0 || mbar_wait_bounded(&bar, 0);
  // one verdict for the block (each thread's wait ran out on its own)
  if (__syncthreads_or(!loaded)) {
    // leave the tile; a second bounded wait lets the copies land first
    if (threadIdx.x == 0) {
      mbar_wait_bounded(&bar, 0);
      atomicOr(err, ERR_TIMEOUT);
    }
    return;
  }
  for (int k = threadIdx.x; k < n; k += NT) {
    const int c = cell_of_word(k < ns ? su[k].w : __ldg(&src.u[b + k].w));
    if (c >= 0) atomicAdd(&cursor[c], 1);
  }
  __syncthreads();
  int nvalid;
  {
    int v[CPT], sum = 0;
#pragma unroll
    for (int e = 0; e < CPT; ++e) {
      v[e] = cursor[threadIdx.x * CPT + e];
      sum += v[e];
    }
    int pre = block_exclusive_scan<NT>(sum, nvalid, swarp);
#pragma unroll
    for (int e = 0; e < CPT; ++e) {
      cursor[threadIdx.x * CPT + e] = pre;
      pre += v[e];
    }
  }
  __syncthreads();
  if (n <= S) {
    for (int k = threadIdx.x; k < n; k += NT) {
      const int c = cell_of_word(su[k].w);
      if (c >= 0) perm[tile_slot(atomicAdd(&cursor[c], 1), nvalid)] = (unsigned short)k;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nvalid; j += NT) {
      const int k = perm[j];
      dst.u[b + j] = su[k];
      dst.xy[b + j] = sxy[k];
    }
  } else {
    for (int k = threadIdx.x; k < n; k += NT) {
      float4 u;
      float2 xy;
      if (k < ns) {
        u = su[k];
        xy = sxy[k];
      } else {
        u = __ldg(&src.u[b + k]);
        xy = __ldg(&src.xy[b + k]);
      }
      const int c = cell_of_word(u.w);
      if (c < 0) continue;
      const int slot = tile_slot(atomicAdd(&cursor[c], 1), nvalid);
      dst.u[b + slot] = u;
      dst.xy[b + slot] = xy;
    }
  }
  if (threadIdx.x == 0) np[t] = nvalid;
}

// The same sort without staging, for runs that share the GPU with others
// (batches): every thread keeps two particles' loads in flight, the count
// and the scatter read global memory, and a block needs 4 KB of shared
// memory, so sort blocks sit beside the other runs' kernels.
template <int NT>
__global__ void __launch_bounds__(NT, 2048 / NT) k_cellsort_direct(Particles src, Particles dst, const int *off,
                                                                    int *np, LayoutConst L) {
  constexpr int MAXC = 1024, ILP = 2, CPT = MAXC / NT;
  __shared__ int cursor[MAXC];
  __shared__ int swarp[NT / 32];
  const int t = blockIdx.x;
  const int ncell = L.TX * L.TY;
  const int cx0 = (t % L.ntx) * L.TX, cy0 = (t / L.ntx) * L.TY;
  const int n = np[t];
  const long long b = off[t];
  for (int c = threadIdx.x; c < MAXC; c += NT) cursor[c] = 0;
  __syncthreads();
  auto cell_of_word = [&](float w) {  // -1 for a hole
    const unsigned u = (unsigned)__float_as_int(w);
    if (u == kHole) return -1;
    const int c = ((int)(u & 0xffffu) - cx0) + ((int)(u >> 16) - cy0) * L.TX;
    return min(max(c, 0), ncell - 1);
  };
  const float hole = __int_as_float((int)kHole);
  for (int k0 = threadIdx.x; k0 < n; k0 += ILP * NT) {
    float w[ILP];
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int k = k0 + q * NT;
      w[q] = (k < n) ? __ldg(&src.u[b + k].w) : hole;
    }
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int c = cell_of_word(w[q]);
      if (c >= 0) atomicAdd(&cursor[c], 1);
    }
  }
  __syncthreads();
  int nvalid;
  {
    int v[CPT], sum = 0;
#pragma unroll
    for (int e = 0; e < CPT; ++e) {
      v[e] = cursor[threadIdx.x * CPT + e];
      sum += v[e];
    }
    int pre = block_exclusive_scan<NT>(sum, nvalid, swarp);
#pragma unroll
    for (int e = 0; e < CPT; ++e) {
      cursor[threadIdx.x * CPT + e] = pre;
      pre += v[e];
    }
  }
  __syncthreads();
  for (int k0 = threadIdx.x; k0 < n; k0 += ILP * NT) {
    float4 u[ILP];
    float2 xy[ILP];
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int k = k0 + q * NT;
      if (k < n) {
        u[q] = __ldg(&src.u[b + k]);
        xy[q] = __ldg(&src.xy[b + k]);
      } else {
        u[q].w = hole;
      }
    }
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int c = cell_of_word(u[q].w);
      if (c < 0) continue;
      const int slot = tile_slot(atomicAdd(&cursor[c], 1), nvalid);
      dst.u[b + slot] = u[q];
      dst.xy[b + slot] = xy[q];
    }
  }
  if (threadIdx.x == 0) np[t] = nvalid;
}

// appends a list to the tiles in place (moving-window injection); overflow
// goes to the spill list that the next push processes
__global__ void k_append_list(Particles list, int n, Particles buf, TileSet T, Spill S, LayoutConst L,
                              int *err) {
  int errbits = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const PRec r = load_particle(list, k);
    if (r.ix < 0 || r.ix >= L.nx || r.iy < 0 || r.iy >= L.ny) {
      errbits |= ERR_ESCAPE;
      continue;
    }
    const int t = tile_of(r.ix, r.iy, L);
    const int s = atomicAdd(&T.np[t], 1);
    if (s < T.cap[t])
      store_particle(buf, (long long)T.off[t] + s, r);
    else
      spill_particle(S, &errbits, r);
  }
  if (errbits) atomicOr(err, errbits);
}

__global__ void k_clamp_counts(int *np, const int *cap, int ntiles) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    np[t] = min(np[t], cap[t]);
}

// tiles + spill -> AoS records in tile order (download), holes dropped;
// dst_off from the tiles' particle counts (one CTA of 256 threads per tile)
__global__ void __launch_bounds__(256) k_gather_aos(Particles buf, const int *off, const int *np,
                                                    const long long *dst_off, int *aos, int ntiles) {
  __shared__ int swarp[8];
  const int t = blockIdx.x;
  if (t >= ntiles) return;
  const int n = np[t];
  const long long a = off[t], d = dst_off[t];
  int placed = 0;
  for (int k0 = 0; k0 < n; k0 += 256) {
    const int k = k0 + threadIdx.x;
    const bool f = k < n && !is_hole(buf, a + k);
    int tot;
    const int pre = block_exclusive_scan<256>(f ? 1 : 0, tot, swarp);
    if (f) {
      int *r = aos + 7LL * (d + placed + pre);
      const PRec q = load_particle(buf, a + k);
      r[0] = q.ix;
      r[1] = q.iy;
      r[2] = __float_as_int(q.x);
      r[3] = __float_as_int(q.y);
      r[4] = __float_as_int(q.ux);
      r[5] = __float_as_int(q.uy);
      r[6] = __float_as_int(q.uz);
    }
    placed += tot;
  }
}

__global__ void k_list_to_aos(Particles list, const int *n_ptr, int n_cap, int *aos, long long d0) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int *r = aos + 7LL * (d0 + k);
    const PRec q = load_particle(list, k);
    r[0] = q.ix;
    r[1] = q.iy;
    r[2] = __float_as_int(q.x);
    r[3] = __float_as_int(q.y);
    r[4] = __float_as_int(q.ux);
    r[5] = __float_as_int(q.uy);
    r[6] = __float_as_int(q.uz);
  }
}

// charge density of the particles of a tile set / list on an (nx+1)(ny+1)
// grid (spec_deposit_charge, particles.c:1289-1309)
__global__ void k_charge_tiles(Particles buf, const int *off, const int *np, float *rho, int nrow, float q,
                               int ntiles) {
  const int t = blockIdx.x;
  if (t >= ntiles) return;
  const int n = np[t];
  const long long a = off[t];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    if (is_hole(buf, a + k)) continue;
    const PRec r = load_particle(buf, a + k);
    const int c = r.ix + nrow * r.iy;
    const float w1 = r.x, w2 = r.y;
    atomicAdd(&rho[c], (1.0f - w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + 1], (w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + nrow], (1.0f - w1) * (w2) * q);
    atomicAdd(&rho[c + 1 + nrow], (w1) * (w2) * q);
  }
}

__global__ void k_charge_list(Particles list, const int *n_ptr, int n_cap, float *rho, int nrow, float q) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const PRec r = load_particle(list, k);
    const int c = r.ix + nrow * r.iy;
    const float w1 = r.x, w2 = r.y;
    atomicAdd(&rho[c], (1.0f - w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + 1], (w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + nrow], (1.0f - w1) * (w2) * q);
    atomicAdd(&rho[c + 1 + nrow], (w1) * (w2) * q);
  }
}

// ---------------------------------------------------------------------------
// device-side loading (spec_set_x / spec_set_u, particles.c:85-354): the
// ppc lattice of every cell, kept where the density profile includes it
// (uniform, step, slab as spec_set_x tests the lattice points), thermal
// momenta from a counter-based generator, each cell's mean momentum
// removed and the fluid drift added; written straight into the tiles in
// cell order.  One thread per cell: the cell's particles and its mean stay
// in that thread.
// ---------------------------------------------------------------------------

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): 10 rounds of the 4x32 multiply-xor bijection
// keyed by a 64-bit key, on a 128-bit counter
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  constexpr unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  constexpr unsigned W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const unsigned hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// uniform in (0, 1) from 32 random bits
__device__ __forceinline__ float u01(unsigned v) { return ((v >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// three standard normal deviates (Box-Muller on two pairs of uniforms)
__device__ __forceinline__ void normal3(uint4 r, float &a, float &b, float &c) {
  const float r0 = sqrtf(-2.0f * logf(u01(r.x))), r1 = sqrtf(-2.0f * logf(u01(r.z)));
  float s0, c0, s1, c1;
  sincospif(2.0f * u01(r.y), &s0, &c0);
  sincospif(2.0f * u01(r.w), &s1, &c1);
  a = r0 * c0;
  b = r0 * s0;
  c = r1 * c1;
}

__global__ void __launch_bounds__(256) k_init_tiles(Particles buf, const int *off, const int *colpts,
                                                    const unsigned *colmask, InitConst I, LayoutConst L) {
  const int t = blockIdx.x;
  const int tx = t % L.ntx, ty = t / L.ntx;
  const int cx0 = tx * L.TX, cy0 = ty * L.TY;
  const int wx = min(L.TX, L.nx - cx0), wy = min(L.TY, L.ny - cy0);  // cells of this (maybe partial) tile
  // particles per cell column of the tile, and their prefix
  __shared__ int spre[65];
  if (threadIdx.x == 0) {
    int a = 0;
    for (int li = 0; li < wx; ++li) {
      spre[li] = a;
      a += colpts[cx0 + li] * I.ppcy;
    }
    spre[wx] = a;
  }
  __syncthreads();
  const int row = spre[wx];  // particles in one row of cells of the tile
  const int ntile = row * wy;
  const long long base = off[t];
  for (int cell = threadIdx.x; cell < L.TX * L.TY; cell += blockDim.x) {
    const int li = cell % L.TX, lj = cell / L.TX;
    if (li >= wx || lj >= wy) continue;
    const int i = cx0 + li, j = cy0 + lj;
    const int nc = colpts[i] * I.ppcy;
    if (nc == 0) continue;
    // cell order inside the tile: local index li + lj * TX; position p of
    // that order is stored at slot tile_slot(p, ntile)
    const int o = lj * row + spre[li];
    const unsigned mask = colmask[i];
    float mx = 0.f, my = 0.f, mz = 0.f;
    int m = 0;
    const unsigned long long cid = (unsigned long long)j * L.nx + i;
    for (int b = 0; b < I.ppcy; ++b)
      for (int a = 0; a < I.ppcx; ++a) {
        if (!(mask >> a & 1)) continue;
        const uint4 r = philox4x32_10(make_uint4((unsigned)cid, (unsigned)(cid >> 32), (unsigned)(b * I.ppcx + a), 0u),
                                      make_uint2(I.seed_lo, I.seed_hi));
        float n0, n1, n2;
        normal3(r, n0, n1, n2);
        const float ux = I.uth[0] * n0, uy = I.uth[1] * n1, uz = I.uth[2] * n2;
        mx += ux;
        my += uy;
        mz += uz;
        store_particle(buf, base + tile_slot(o + m, ntile), i, j, I.hx * (a + 0.5f), I.hy * (b + 0.5f), ux, uy,
                       uz);
        ++m;
      }
    // remove the cell's mean momentum, add the fluid drift (particles.c:102-146)
    const float inv = 1.0f / m;
    mx *= inv;
    my *= inv;
    mz *= inv;
    for (int k = 0; k < m; ++k) {
      const long long q = base + tile_slot(o + k, ntile);
      PRec r = load_particle(buf, q);
      store_particle(buf, q, r.ix, r.iy, r.x, r.y, r.ux - mx + I.ufl[0], r.uy - my + I.ufl[1],
                     r.uz - mz + I.ufl[2]);
    }
  }
}

cudaError_t launch_init_tiles(const Particles &buf, const int *off, const int *colpts, const unsigned *colmask,
                              const InitConst &I, const LayoutConst &L, int ntiles, cudaStream_t st) {
  k_init_tiles<<<ntiles, 256, 0, st>>>(buf, off, colpts, colmask, I, L);
  return cudaGetLastError();
}

// phase-space density (spec_deposit_pha, particles.c:1569-1632): the two
// axis quantities of spec_pha_axis (particles.c:1510-1536), linear weights
// onto an n1 x n2 grid, out-of-range cells dropped
__device__ __forceinline__ float pha_quant(const PRec &r, int q, const PhaConst &P) {
  switch (q) {
    case 1: return (r.x + r.ix) * P.dx;
    case 2: return (r.y + r.iy) * P.dy;
    case 4: return r.ux;
    case 5: return r.uy;
    default: return r.uz;
  }
}

__device__ __forceinline__ void pha_add(float *buf, const PRec &r, const PhaConst &P) {
  const float nx1 = (pha_quant(r, P.q1, P) - P.x1min) * P.rdx1;
  const float nx2 = (pha_quant(r, P.q2, P) - P.x2min) * P.rdx2;
  const int i1 = (int)(nx1 + 0.5f), i2 = (int)(nx2 + 0.5f);
  const float w1 = nx1 - i1 + 0.5f, w2 = nx2 - i2 + 0.5f;
  const int idx = i1 + P.n1 * i2;
  const bool a0 = i1 >= 0 && i1 < P.n1, a1 = i1 + 1 >= 0 && i1 + 1 < P.n1;
  if (i2 >= 0 && i2 < P.n2) {
    if (a0) atomicAdd(&buf[idx], (1.0f - w1) * (1.0f - w2) * P.q);
    if (a1) atomicAdd(&buf[idx + 1], w1 * (1.0f - w2) * P.q);
  }
  if (i2 + 1 >= 0 && i2 + 1 < P.n2) {
    if (a0) atomicAdd(&buf[idx + P.n1], (1.0f - w1) * w2 * P.q);
    if (a1) atomicAdd(&buf[idx + P.n1 + 1], w1 * w2 * P.q);
  }
}

__global__ void k_pha_tiles(Particles buf, const int *off, const int *np, int ntiles, float *pha, PhaConst P) {
  const int t = blockIdx.x;
  if (t >= ntiles) return;
  const int n = np[t];
  const long long a = off[t];
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    if (!is_hole(buf, a + k)) pha_add(pha, load_particle(buf, a + k), P);
}

__global__ void k_pha_list(Particles list, const int *n_ptr, int n_cap, float *pha, PhaConst P) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    pha_add(pha, load_particle(list, k), P);
}

cudaError_t launch_phasespace(const Particles &buf, const int *off, const int *np, int ntiles, const Particles &spill,
                              const int *spill_cnt, int spill_cap, float *pha, const PhaConst &P, cudaStream_t st) {
  k_pha_tiles<<<ntiles, 256, 0, st>>>(buf, off, np, ntiles, pha, P);
  k_pha_list<<<64, 256, 0, st>>>(spill, spill_cnt, spill_cap, pha, P);
  return cudaGetLastError();
}

// boundary corrections of the charge grid (particles.c:1311-1321)
__global__ void k_charge_fold(float *rho, int nx, int ny, int mw) {
  const int nrow = nx + 1;
  if (blockIdx.x == 0) {
    if (!mw)
      for (int j = threadIdx.x; j < ny + 1; j += blockDim.x) rho[j * nrow] += rho[nx + j * nrow];
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < nx + 1; i += blockDim.x) rho[i] += rho[i + ny * nrow];
}

// sum of the per-tile kinetic-energy partials in a fixed order
__global__ void k_sum_energy(const double *tiles, int ntiles, const double *extra, double *out, float scale_q_mq,
                             float dx, float dy, int det) {
  __shared__ double sred[8];
  double s = 0;
  for (int t = threadIdx.x; t < ntiles; t += 256) s += tiles[t];
  s = block_sum_double<256>(s, sred);
  if (threadIdx.x == 0) {
    if (det) {
      const long long *w = reinterpret_cast<const long long *>(extra);
      s += efix_join(w[0], w[1]);
    } else {
      s += *extra;
    }
    // spec->energy = q * m_q * energy * dx * dy  (particles.c:1231)
    *out = scale_q_mq * s * dx * dy;
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
bool tile_supported(int TX, int TY) {
  return (TX == 16 && TY == 16) || (TX == 8 && TY == 8) || (TX == 16 && TY == 8) || (TX == 32 && TY == 16) ||
         (TX == 32 && TY == 32) || (TX == 8 && TY == 16) || (TX == 16 && TY == 32);
}

cudaError_t launch_push_tiles(const PushLaunch &a, cudaStream_t st) {
  if (a.det) return a.fast ? launch_push_tiles_fast_det(a, st) : launch_push_tiles_exact_det(a, st);
  return a.fast ? launch_push_tiles_fast(a, st) : launch_push_tiles_exact(a, st);
}

cudaError_t launch_push_spill(const float *EB, float *J, const FixedJ &fj, const Grid &G, const Particles &sin,
                              const int *sin_cnt, int sin_cap, const Spill &S, double *ekin, int *err,
                              const PushConst &C, int nblocks, int fast, int det, cudaStream_t st) {
  auto f = det ? (fast ? launch_push_spill_fast_det : launch_push_spill_exact_det)
               : (fast ? launch_push_spill_fast : launch_push_spill_exact);
  return f(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C, nblocks, st);
}

__global__ void k_fixed_to_float(const unsigned long long *src, float *dst, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = (float)((double)(long long)src[k] / kJFixScale);
}

__global__ void k_float_to_fixed(const float *src, unsigned long long *dst, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = (unsigned long long)__double2ll_rn((double)src[k] * kJFixScale);
}

cudaError_t launch_fixed_to_float(const unsigned long long *src, float *dst, size_t n, cudaStream_t st) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_fixed_to_float<<<blocks, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_float_to_fixed(const float *src, unsigned long long *dst, size_t n, cudaStream_t st) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_float_to_fixed<<<blocks, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

// staging room: the cursors and 26 bytes a particle within 227 KB (and
// slots that fit 16 bits)
constexpr int kSortStageMax = 8704;
constexpr int kSortStageBytes = (int)(sizeof(float4) + sizeof(float2) + sizeof(unsigned short));

cudaError_t launch_cellsort(const Particles &src, const Particles &dst, const int *off, int *np,
                            const LayoutConst &L, int ntiles, int max_n, int *err, cudaStream_t st) {
  if (max_n <= 0) {
    k_cellsort_direct<ZC_SORT_NT><<<ntiles, ZC_SORT_NT, 0, st>>>(src, dst, off, np, L);
    return cudaGetLastError();
  }
  // the shared-memory opt-in, once per device
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(opted.load() & bit)) {
    e = cudaFuncSetAttribute(k_cellsort<ZC_SORT_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             1024 * (int)sizeof(int) + kSortStageMax * kSortStageBytes);
    if (e != cudaSuccess) return e;
    opted.fetch_or(bit);
  }
  const int S = std::min(max_n, kSortStageMax);
  const size_t smem = 1024 * sizeof(int) + (size_t)S * kSortStageBytes;
  k_cellsort<ZC_SORT_NT><<<ntiles, ZC_SORT_NT, smem, st>>>(src, dst, off, np, L, S, err);
  return cudaGetLastError();
}

cudaError_t launch_count_valid(const Particles &buf, const int *off, const int *np, int *cnt, int ntiles,
                               cudaStream_t st) {
  k_count_valid<<<ntiles, 256, 0, st>>>(buf, off, np, cnt);
  return cudaGetLastError();
}

cudaError_t launch_settle(const Particles &buf, const TileSet &T, const Outbox &O, const Spill &S, int *err,
                          int ntx, int nty, int mw, cudaStream_t st) {
  k_migrate<256><<<ntx * nty, 256, 0, st>>>(buf, T, O, S, err, ntx, nty, mw);
  return cudaGetLastError();
}

__global__ void k_inject_column(Particles list, ColumnInject C) {
  const int n = C.ny * C.cnt;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int j = t / C.cnt, q = t - j * C.cnt;
    store_particle(list, t, C.ix, j, C.px[q], C.py[q], C.ux, C.uy, C.uz);
  }
}

cudaError_t launch_inject_column(const Particles &list, const ColumnInject &C, cudaStream_t st) {
  const int n = C.ny * C.cnt;
  if (n <= 0) return cudaSuccess;
  k_inject_column<<<(n + 255) / 256, 256, 0, st>>>(list, C);
  return cudaGetLastError();
}

cudaError_t launch_stage_to_list(const void *aos, int n, const Particles &list, int *cell_cnt,
                                 const LayoutConst &L, int *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  k_stage_to_list<<<nb, 256, 0, st>>>(reinterpret_cast<const int *>(aos), n, list, cell_cnt, L, err);
  return cudaGetLastError();
}

cudaError_t launch_cell_starts(int *cell, int *cnt, const LayoutConst &L, int ntiles, cudaStream_t st) {
  k_cell_starts<<<ntiles, 1024, 0, st>>>(cell, cnt, L);
  return cudaGetLastError();
}

cudaError_t launch_scatter_sorted(const Particles &list, int n, const Particles &dst, const int *off,
                                  const int *cnt, int *cell_pos, const LayoutConst &L, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = (int)std::min<long long>((n + 255) / 256, 152 * 8);
  k_scatter_sorted<<<nb, 256, 0, st>>>(list, n, dst, off, cnt, cell_pos, L);
  return cudaGetLastError();
}

cudaError_t launch_count_list(const Particles &list, const int *n_ptr, int n_cap, int *cnt, const LayoutConst &L,
                              cudaStream_t st) {
  k_count_list<<<256, 256, 0, st>>>(list, n_ptr, n_cap, cnt, L);
  return cudaGetLastError();
}

cudaError_t launch_copy_tiles(const Particles &src, const int *off_old, const int *np_old, const Particles &dst,
                              const int *off_new, int *fill, int ntiles, cudaStream_t st) {
  k_copy_tiles<<<ntiles, 256, 0, st>>>(src, off_old, np_old, dst, off_new, fill);
  return cudaGetLastError();
}

cudaError_t launch_scatter_list(const Particles &list, const int *n_ptr, int n_cap, const Particles &dst,
                                const int *off, const int *cap, int *fill, const LayoutConst &L, int *err,
                                cudaStream_t st) {
  k_scatter_list<<<512, 256, 0, st>>>(list, n_ptr, n_cap, dst, off, cap, fill, L, err);
  return cudaGetLastError();
}

cudaError_t launch_append_list(const Particles &list, int n, const Particles &buf, const TileSet &T,
                               const Spill &S, const LayoutConst &L, int *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_append_list<<<(n + 255) / 256, 256, 0, st>>>(list, n, buf, T, S, L, err);
  k_clamp_counts<<<(T.ntiles + 255) / 256, 256, 0, st>>>(T.np, T.cap, T.ntiles);
  return cudaGetLastError();
}

cudaError_t launch_gather_aos(const Particles &buf, const int *off, const int *np, const long long *dst_off,
                              int *aos, int ntiles, cudaStream_t st) {
  k_gather_aos<<<ntiles, 256, 0, st>>>(buf, off, np, dst_off, aos, ntiles);
  return cudaGetLastError();
}

cudaError_t launch_list_to_aos(const Particles &list, const int *n_ptr, int n_cap, int *aos, long long d0,
                               cudaStream_t st) {
  k_list_to_aos<<<256, 256, 0, st>>>(list, n_ptr, n_cap, aos, d0);
  return cudaGetLastError();
}

cudaError_t launch_charge(const Particles &buf, const int *off, const int *np, int ntiles, const Particles &spill,
                          const int *spill_cnt, int spill_cap, float *rho, int nx, int ny, float q, int mw,
                          cudaStream_t st) {
  k_charge_tiles<<<ntiles, 256, 0, st>>>(buf, off, np, rho, nx + 1, q, ntiles);
  k_charge_list<<<64, 256, 0, st>>>(spill, spill_cnt, spill_cap, rho, nx + 1, q);
  k_charge_fold<<<1, 256, 0, st>>>(rho, nx, ny, mw);
  return cudaGetLastError();
}

cudaError_t launch_sum_energy(const double *tiles, int ntiles, const double *extra, double *out, float q_mq,
                              float dx, float dy, int det, cudaStream_t st) {
  k_sum_energy<<<1, 256, 0, st>>>(tiles, ntiles, extra, out, q_mq, dx, dy, det);
  return cudaGetLastError();
}

}  // namespace zc
