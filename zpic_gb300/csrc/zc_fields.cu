// zc_fields.cu -- grid kernels of libzpic_cuda (sm_103a): current guard-cell
// fold and digital filtering, the fused Yee field advance, field guard
// cells, external fields, moving window, laser launch and FP64 energies.
//
// Compiled with -fmad=false: every cell is computed with the same float32
// operations, in the same order, as the reference (em2d/current.c,
// em2d/emf.c), so from the same inputs these kernels return the same bits.
// All of them are HBM-bound stencils; none is a contraction.
#include <math.h>

#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {

__device__ __forceinline__ size_t gidx(const Grid &G, int c, int bx, int by) {
  return c * G.plane + (size_t)by * G.pitch + bx;
}

// ---------------------------------------------------------------------------
// layout conversion: reference float3 AoS buffers <-> SoA planes
// ---------------------------------------------------------------------------
__global__ void k_aos_to_planes(const float *aos, float *planes, Grid G, int ncomp) {
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int n = gx * gy;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int bx = k % gx, by = k / gx;
    for (int c = 0; c < ncomp; ++c) planes[gidx(G, c, bx, by)] = aos[(size_t)k * ncomp + c];
  }
}

__global__ void k_planes_to_aos(const float *planes, float *aos, Grid G, int ncomp) {
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int n = gx * gy;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int bx = k % gx, by = k / gx;
    for (int c = 0; c < ncomp; ++c) aos[(size_t)k * ncomp + c] = planes[gidx(G, c, bx, by)];
  }
}

// ---------------------------------------------------------------------------
// current guard-cell fold (current_update_gc, em2d/current.c:118-159)
// ---------------------------------------------------------------------------
__global__ void k_fold_x(float *J, Grid G) {
  const int by = blockIdx.x * blockDim.x + threadIdx.x;  // every buffer row
  if (by >= G.ny + 3) return;
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b) {  // cells -1, 0, 1 receive nx-1, nx, nx+1
      const size_t lo = gidx(G, c, b, by), hi = gidx(G, c, G.nx + b, by);
      const float v = J[lo] + J[hi];
      J[lo] = v;
      J[hi] = v;
    }
}

__global__ void k_fold_y(float *J, Grid G) {
  const int bx = blockIdx.x * blockDim.x + threadIdx.x;  // every buffer column
  if (bx >= G.nx + 3) return;
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b) {
      const size_t lo = gidx(G, c, bx, b), hi = gidx(G, c, bx, G.ny + b);
      const float v = J[lo] + J[hi];
      J[lo] = v;
      J[hi] = v;
    }
}

// ---------------------------------------------------------------------------
// one [sa, sb, sa] filter tap (kernel_x / kernel_y, em2d/current.c:316-413)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float f3pt(float sa, float sb, float l, float m, float u) {
  return sa * l + sb * m + sa * u;
}

// ---------------------------------------------------------------------------
// all filter passes along one axis in one kernel.  Passes along x act on
// every interior row independently: a CTA loads its row (guards included)
// into shared memory, runs the passes there -- refreshing the periodic x
// guards after each pass unless the window moves, as kernel_x does -- and
// writes the row back in place.  Passes along y are periodic convolutions
// over the interior rows (kernel_y refreshes the y guards after each pass),
// except that the first pass reads the y guard rows as they are (the x
// passes leave them at their pre-filter values): a CTA takes a strip of 32
// columns and ROWS rows plus one halo row per pass on each side, runs the
// passes in shared memory and writes its rows (and the y guard rows they
// feed) out of place.  Every cell sees the same float
// operations in the same order as with one kernel per pass.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_smooth_x_all(float *J, Grid G, SmoothPasses P, int mw) {
  extern __shared__ float srow[];  // [2][gx]: one component of one row
  const int gx = G.nx + 3;
  const int by = blockIdx.x + 1;   // interior row
  const int c = blockIdx.y;        // component
  // asynchronous copies: every load of the row in flight at once
  for (int bx = threadIdx.x; bx < gx; bx += blockDim.x) cp_async4_zfill(srow + bx, J + gidx(G, c, bx, by), true);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  int cur = 0;
  for (int p = 0; p < P.n; ++p) {
    const float sa = P.sa[p], sb = P.sb[p];
    const float *r = srow + cur * gx;
    float *o = srow + (1 - cur) * gx;
    for (int bx = threadIdx.x; bx < gx; bx += blockDim.x) {
      float v;
      if (bx >= 1 && bx <= G.nx) v = f3pt(sa, sb, r[bx - 1], r[bx], r[bx + 1]);
      else if (mw) v = r[bx];
      else {
        const int s = (bx == 0) ? G.nx : bx - G.nx;  // guard <- filtered interior value
        v = f3pt(sa, sb, r[s - 1], r[s], r[s + 1]);
      }
      o[bx] = v;
    }
    __syncthreads();
    cur = 1 - cur;
  }
  for (int bx = threadIdx.x; bx < gx; bx += blockDim.x) J[gidx(G, c, bx, by)] = srow[cur * gx + bx];
}

constexpr int kSmoothYRows = 64;   // interior rows per CTA
constexpr int kSmoothYCols = 32;   // columns per CTA (one warp across)

__global__ void __launch_bounds__(256) k_smooth_y_all(const float *Jin, float *Jout, Grid G, SmoothPasses P) {
  extern __shared__ float sbuf[];  // [2][ROWS + 2H][COLS], then guard rows [2][COLS]; one component
  const int H = P.n;
  const int R = kSmoothYRows + 2 * H;
  constexpr int W = kSmoothYCols;
  const int gx = G.nx + 3;
  const int c = blockIdx.z;                                  // component
  const int cc = threadIdx.x & 31, r0 = threadIdx.x >> 5;   // column, first row of this thread
  const int bx = blockIdx.x * W + cc;
  const bool col_ok = bx < gx;
  const bool filt = bx >= 1 && bx <= G.nx;                   // only interior columns are filtered
  const int j0 = blockIdx.y * kSmoothYRows;                  // first interior row of the strip
  float *glo = sbuf + 2 * R * W, *ghi = glo + W;             // y guard rows -1 and ny as stored
  if (r0 == 0) {
    cp_async4_zfill(glo + cc, col_ok ? Jin + gidx(G, c, bx, 0) : Jin, col_ok);
    cp_async4_zfill(ghi + cc, col_ok ? Jin + gidx(G, c, bx, G.ny + 1) : Jin, col_ok);
  }
  // rows j0-H .. j0+ROWS+H-1, wrapped periodically over the interior rows
  for (int rr = r0; rr < R; rr += 8) {
    int j = (j0 - H + rr) % G.ny;
    if (j < 0) j += G.ny;
    cp_async4_zfill(sbuf + rr * W + cc, col_ok ? Jin + gidx(G, c, bx, j + 1) : Jin, col_ok);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  int cur = 0;
  for (int p = 0; p < P.n; ++p) {
    const float sa = P.sa[p], sb = P.sb[p];
    const float *in = sbuf + cur * R * W;
    float *out = sbuf + (1 - cur) * R * W;
    for (int rr = r0; rr < R; rr += 8) {
      bool lo_guard = false, hi_guard = false;
      if (p == 0) {
        int jm = (j0 - H + rr) % G.ny;
        if (jm < 0) jm += G.ny;
        lo_guard = (jm == 0);
        hi_guard = (jm == G.ny - 1);
      }
      const bool inside = rr > p && rr < R - 1 - p;
      const int k = rr * W + cc;
      float v = in[k];
      if (inside && filt) {
        const float lo = lo_guard ? glo[cc] : in[k - W];
        const float hi = hi_guard ? ghi[cc] : in[k + W];
        v = f3pt(sa, sb, lo, in[k], hi);
      }
      out[k] = v;
    }
    __syncthreads();
    cur = 1 - cur;
  }
  if (!col_ok) return;
  const float *res = sbuf + cur * R * W;
  for (int rr = r0; rr < kSmoothYRows; rr += 8) {
    const int j = j0 + rr;
    if (j >= G.ny) break;
    const float v = res[(rr + H) * W + cc];
    Jout[gidx(G, c, bx, j + 1)] = v;
    // y guard rows are periodic copies of the filtered interior rows
    if (j == G.ny - 1) Jout[gidx(G, c, bx, 0)] = v;
    if (j < 2) Jout[gidx(G, c, bx, G.ny + 1 + j)] = v;
  }
}

// Both axes in one pass over J (the x passes of every row of the strip, its
// halo rows included, then the y passes), for the common case of filtering
// along both: the rows are filtered along x in shared memory with a halo of
// one column per x pass -- periodic images of the interior columns, or with a
// moving window the fixed guard columns -- so that each cell sees exactly the
// float operations of k_smooth_x_all followed by k_smooth_y_all.
__global__ void __launch_bounds__(256, 6) k_smooth_xy_all(const float *Jin, float *Jout, Grid G, SmoothPasses PX,
                                                       SmoothPasses P, int mw) {
  // rows [2][R][XW] (x halo of HX columns each side), guard rows [2][W],
  // interior row index of each tile row (periodic)
  extern __shared__ float sbuf[];
  const int H = P.n, HX = PX.n;
  const int R = kSmoothYRows + 2 * H;
  constexpr int W = kSmoothYCols;
  const int XW = W + 2 * HX;
  const int gx = G.nx + 3;
  const int c = blockIdx.z;
  const int bx0 = blockIdx.x * W;
  const int j0 = blockIdx.y * kSmoothYRows;
  float *glo = sbuf + 2 * R * XW, *ghi = glo + W;
  int *rowj = reinterpret_cast<int *>(ghi + W);
  const int tid = threadIdx.x;
  if (tid < W) {
    const int b = bx0 + tid;
    cp_async4_zfill(glo + tid, b < gx ? Jin + gidx(G, c, b, 0) : Jin, b < gx);
    cp_async4_zfill(ghi + tid, b < gx ? Jin + gidx(G, c, b, G.ny + 1) : Jin, b < gx);
  }
  for (int rr = tid; rr < R; rr += blockDim.x) {
    int jm = (j0 - H + rr) % G.ny;
    rowj[rr] = jm < 0 ? jm + G.ny : jm;
  }
  __syncthreads();
  // k = rr * XW + q walks the tile in steps of the block size
  const int step_r = blockDim.x / XW, step_q = blockDim.x % XW;
  const int n = R * XW;
  {
    int rr = tid / XW, q = tid % XW;
    for (int k = tid; k < n; k += blockDim.x) {
      // buffer column of strip column q: with a moving window the column
      // itself (zero outside the buffer), else its periodic image over the
      // interior columns
      int b = bx0 - HX + q;
      if (!mw && (b < 1 || b > G.nx)) b = ((b - 1) % G.nx + G.nx) % G.nx + 1;
      const bool ok = b >= 0 && b < gx;
      cp_async4_zfill(sbuf + k, ok ? Jin + gidx(G, c, b, rowj[rr] + 1) : Jin, ok);
      q += step_q;
      rr += step_r;
      if (q >= XW) { q -= XW; ++rr; }
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  // x passes (kernel_x): every strip column filtered from its neighbours,
  // except the guard columns of a moving window, which stay as they are;
  // after p passes the columns p .. XW-1-p hold the filtered values
  int cur = 0;
  for (int p = 0; p < HX; ++p) {
    const float sa = PX.sa[p], sb = PX.sb[p];
    const float *in = sbuf + cur * R * XW;
    float *out = sbuf + (1 - cur) * R * XW;
    int q = tid % XW;
    for (int k = tid; k < n; k += blockDim.x) {
      const int b = bx0 - HX + q;
      float v = in[k];
      if (q > 0 && q < XW - 1 && (!mw || (b >= 1 && b <= G.nx))) v = f3pt(sa, sb, in[k - 1], in[k], in[k + 1]);
      out[k] = v;
      q += step_q;
      if (q >= XW) q -= XW;
    }
    __syncthreads();
    cur = 1 - cur;
  }
  // y passes (kernel_y) on the strip's own columns, as k_smooth_y_all
  const int cc = tid & 31, r0 = tid >> 5;
  const int bx = bx0 + cc;
  const bool filt = bx >= 1 && bx <= G.nx;
  for (int p = 0; p < H; ++p) {
    const float sa = P.sa[p], sb = P.sb[p];
    const float *in = sbuf + cur * R * XW + HX;
    float *out = sbuf + (1 - cur) * R * XW + HX;
    for (int rr = r0; rr < R; rr += 8) {
      // the first pass reads the y guard rows as stored
      const int jm = p == 0 ? rowj[rr] : -1;
      const bool inside = rr > p && rr < R - 1 - p;
      const int k = rr * XW + cc;
      float v = in[k];
      if (inside && filt) {
        const float lo = jm == 0 ? glo[cc] : in[k - XW];
        const float hi = jm == G.ny - 1 ? ghi[cc] : in[k + XW];
        v = f3pt(sa, sb, lo, in[k], hi);
      }
      out[k] = v;
    }
    __syncthreads();
    cur = 1 - cur;
  }
  if (bx >= gx) return;
  const float *res = sbuf + cur * R * XW + HX;
  for (int rr = r0; rr < kSmoothYRows; rr += 8) {
    const int j = j0 + rr;
    if (j >= G.ny) break;
    const float v = res[(rr + H) * XW + cc];
    Jout[gidx(G, c, bx, j + 1)] = v;
    if (j == G.ny - 1) Jout[gidx(G, c, bx, 0)] = v;
    if (j < 2) Jout[gidx(G, c, bx, G.ny + 1 + j)] = v;
  }
}

// ---------------------------------------------------------------------------
// fused Yee advance: B half step, E full step, B half step
// (yee_b / yee_e, em2d/emf.c:500-562), one 32 x 16 output tile per CTA.
// E/B and J tiles with their halo arrive by TMA; B1 and E1 live in shared
// memory only; the reference's update ranges (B: cells -1..nx, E: 0..nx+1,
// in buffer coordinates 0..nx+1 and 1..nx+2) are kept exactly so that the
// guard cells evolve as in the reference (they matter with a moving window).
// Out of place: EB in (TMA) -> EB out.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_yee(const __grid_constant__ CUtensorMap tm_eb,
                                             const __grid_constant__ CUtensorMap tm_j, float *EBout, Grid G,
                                             YeeConst Y, int *err) {
  constexpr int BW = kYeeBW, BH = kYeeBH, PL = BW * BH;
  __shared__ __align__(128) float sEB[6 * PL];
  __shared__ __align__(128) float sJ[3 * PL];
  __shared__ __align__(8) uint64_t bar;
  const int bx0 = blockIdx.x * kYeeOX, by0 = blockIdx.y * kYeeOY;
  const int ox = bx0 - 4, oy = by0 - 1;  // buffer coords of smem (0,0)
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, (6 + 3) * PL * 4);
    tma_load_3d(sEB, &tm_eb, ox, oy, 0, &bar);
    tma_load_3d(sJ, &tm_j, ox, oy, 0, &bar);
  }
  if (!mbar_wait_bounded(&bar, 0)) {
    if (threadIdx.x == 0) atomicOr(err, ERR_TIMEOUT);
    if (!mbar_wait_bounded(&bar, 0)) return;  // second bounded wait for the copies in flight
  }

  float *Ex = sEB, *Ey = sEB + PL, *Ez = sEB + 2 * PL;
  float *Bx = sEB + 3 * PL, *By = sEB + 4 * PL, *Bz = sEB + 5 * PL;
  const float *Jx = sJ, *Jy = sJ + PL, *Jz = sJ + 2 * PL;
  const int nx = G.nx, ny = G.ny;

  // B1 on buffer cells [bx0-1, bx0+OX] x [by0-1, by0+OY]
  {
    constexpr int W = kYeeOX + 2, H = kYeeOY + 2;
    for (int k = threadIdx.x; k < W * H; k += blockDim.x) {
      const int bx = bx0 - 1 + k % W, by = by0 - 1 + k / W;
      if (bx < 0 || bx > nx + 1 || by < 0 || by > ny + 1) continue;
      const int s = (by - oy) * BW + (bx - ox);
      Bx[s] += (-Y.cyb * (Ez[s + BW] - Ez[s]));
      By[s] += (Y.cxb * (Ez[s + 1] - Ez[s]));
      Bz[s] += (-Y.cxb * (Ey[s + 1] - Ey[s]) + Y.cyb * (Ex[s + BW] - Ex[s]));
    }
  }
  __syncthreads();
  // E1 on buffer cells [bx0, bx0+OX] x [by0, by0+OY]
  {
    constexpr int W = kYeeOX + 1, H = kYeeOY + 1;
    for (int k = threadIdx.x; k < W * H; k += blockDim.x) {
      const int bx = bx0 + k % W, by = by0 + k / W;
      if (bx < 1 || bx > nx + 2 || by < 1 || by > ny + 2) continue;
      const int s = (by - oy) * BW + (bx - ox);
      Ex[s] += (+Y.cye * (Bz[s] - Bz[s - BW])) - Y.dt * Jx[s];
      Ey[s] += (-Y.cxe * (Bz[s] - Bz[s - 1])) - Y.dt * Jy[s];
      Ez[s] += (+Y.cxe * (By[s] - By[s - 1]) - Y.cye * (Bx[s] - Bx[s - BW])) - Y.dt * Jz[s];
    }
  }
  __syncthreads();
  // B2 on the output tile, then store E1 and B2
  for (int k = threadIdx.x; k < kYeeOX * kYeeOY; k += blockDim.x) {
    const int bx = bx0 + k % kYeeOX, by = by0 + k / kYeeOX;
    if (bx >= nx + 3 || by >= ny + 3) continue;
    const int s = (by - oy) * BW + (bx - ox);
    float bxv = Bx[s], byv = By[s], bzv = Bz[s];
    if (bx <= nx + 1 && by <= ny + 1) {
      bxv += (-Y.cyb * (Ez[s + BW] - Ez[s]));
      byv += (Y.cxb * (Ez[s + 1] - Ez[s]));
      bzv += (-Y.cxb * (Ey[s + 1] - Ey[s]) + Y.cyb * (Ex[s + BW] - Ex[s]));
    }
    EBout[gidx(G, 0, bx, by)] = Ex[s];
    EBout[gidx(G, 1, bx, by)] = Ey[s];
    EBout[gidx(G, 2, bx, by)] = Ez[s];
    EBout[gidx(G, 3, bx, by)] = bxv;
    EBout[gidx(G, 4, bx, by)] = byv;
    EBout[gidx(G, 5, bx, by)] = bzv;
  }
}

// ---------------------------------------------------------------------------
// periodic guard cells of E and B (emf_update_gc, em2d/emf.c:573-637): x
// unless the window moves, y always.  Guards only read interior rows.
// ---------------------------------------------------------------------------
__global__ void k_emf_gc(float *EB, Grid G, int mw) {
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int bx = blockIdx.x * blockDim.x + threadIdx.x;
  const int by = blockIdx.y;
  if (bx >= gx || by >= gy) return;
  const bool gxg = (bx == 0 || bx > G.nx), gyg = (by == 0 || by > G.ny);
  if (!gxg && !gyg) return;
  int sx = bx, sy = by;
  if (gxg && !mw) sx = (bx == 0) ? G.nx : bx - G.nx;
  if (gyg) sy = (by == 0) ? G.ny : by - G.ny;
  if (sx == bx && sy == by) return;
  for (int c = 0; c < 6; ++c) EB[gidx(G, c, bx, by)] = EB[gidx(G, c, sx, sy)];
}

// E_part = E + external, B_part = B + external (emf_update_part_fld,
// em2d/emf.c:838-914); type 0 copies, 1 uniform, 2 grid
__global__ void k_ext_add(const float *EB, float *EBp, const float *extE, const float *extB, int Et, int Bt,
                          float3 E0, float3 B0, Grid G) {
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int bx = blockIdx.x * blockDim.x + threadIdx.x;
  const int by = blockIdx.y;
  if (bx >= gx || by >= gy) return;
  const float e0[3] = {E0.x, E0.y, E0.z}, b0[3] = {B0.x, B0.y, B0.z};
  for (int c = 0; c < 6; ++c) {
    const int t = (c < 3) ? Et : Bt;
    const size_t k = gidx(G, c, bx, by);
    float v = EB[k];
    if (t == 1) v += (c < 3) ? e0[c] : b0[c - 3];
    else if (t == 2) v += (c < 3) ? extE[gidx(G, c, bx, by)] : extB[gidx(G, c - 3, bx, by)];
    EBp[k] = v;
  }
}

// moving window: fields shift left one cell, right-most columns zeroed
// (emf_move_window, em2d/emf.c:648-675); out of place
__global__ void k_window_shift(const float *EBin, float *EBout, Grid G) {
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int bx = blockIdx.x * blockDim.x + threadIdx.x;
  const int by = blockIdx.y;
  if (bx >= gx || by >= gy) return;
  for (int c = 0; c < 6; ++c)
    EBout[gidx(G, c, bx, by)] = (bx < G.nx) ? EBin[gidx(G, c, bx + 1, by)] : 0.0f;
}

// ---------------------------------------------------------------------------
// field energy per component (emf_get_energy, em2d/emf.c:729-750): float
// squares as in the reference, Kahan-compensated per thread, FP64 across
// threads and blocks, partials summed in a fixed order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_emf_energy_partial(const float *EB, Grid G, double *partial) {
  __shared__ double sred[8];
  float s[6] = {0, 0, 0, 0, 0, 0}, cc[6] = {0, 0, 0, 0, 0, 0};
  // interior rows over the blocks, interior columns over the threads: no
  // index division, coalesced rows
  for (int by = blockIdx.x + 1; by <= G.ny; by += gridDim.x) {
    const size_t row = (size_t)by * G.pitch;
    for (int bx = threadIdx.x + 1; bx <= G.nx; bx += blockDim.x) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float f = EB[c * G.plane + row + bx];
        const float y = f * f - cc[c];
        const float t = s[c] + y;
        cc[c] = (t - s[c]) - y;
        s[c] = t;
      }
    }
  }
  for (int c = 0; c < 6; ++c) {
    const double v = block_sum_double<256>((double)s[c] - (double)cc[c], sred);
    if (threadIdx.x == 0) partial[blockIdx.x * 6 + c] = v;
  }
}

__global__ void k_emf_energy_final(const double *partial, int nblocks, double *out, float dx, float dy) {
  if (threadIdx.x < 6) {
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += partial[b * 6 + threadIdx.x];
    out[threadIdx.x] = s * (0.5 * dx * dy);
  }
}

// ---------------------------------------------------------------------------
// laser launch (emf_add_laser, em2d/emf.c:158-350): same double-precision
// library calls on float arguments as the reference
// ---------------------------------------------------------------------------
__device__ float laser_env(const LaserConst &L, float z) {
  const double half_pi = 1.57079632679489661923132169163975144;
  if (z > L.start) return 0.0f;
  if (z > L.start - L.rise) {
    float u = z - L.start;
    float e = sin(half_pi * u / L.rise);
    return e * e;
  }
  if (z > L.start - (L.rise + L.flat)) return 1.0f;
  if (z > L.start - (L.rise + L.flat + L.fall)) {
    float u = z - (L.start - L.rise - L.flat - L.fall);
    float e = sin(half_pi * u / L.fall);
    return e * e;
  }
  return 0.0f;
}

__device__ float laser_gauss(const LaserConst &L, float zpos, float r) {
  float z = zpos - L.focus;
  float zr = L.omega0 * (L.W0 * L.W0) / 2;
  float r2 = r * r;
  float curv = r2 * z / (zr * zr + z * z);
  float w2r = (zr * zr) / (zr * zr + z * z);
  float gouy = atan2((double)z, (double)zr);
  return sqrt(sqrt((double)w2r)) * exp((double)(-r2 * w2r / (L.W0 * L.W0))) *
         cos((double)(L.omega0 * (z + curv) - gouy));
}

__global__ void k_laser_fields(float *EB, Grid G, LaserConst L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= G.nx || j >= G.ny) return;
  const float amp = L.omega0 * L.a0;
  const float cp = cos((double)L.polarization), sp = sin((double)L.polarization);
  const float z = i * L.dx, z2 = z + L.dx / 2;
  const float a = amp * laser_env(L, z), a2 = amp * laser_env(L, z2);
  const int bx = i + 1, by = j + 1;
  float *Ey = &EB[gidx(G, 1, bx, by)], *Ez = &EB[gidx(G, 2, bx, by)];
  float *By = &EB[gidx(G, 4, bx, by)], *Bz = &EB[gidx(G, 5, bx, by)];
  if (L.type == 0) {
    const float k = L.omega0;
    *Ey += +a * cos((double)(k * z)) * cp;
    *Ez += +a * cos((double)(k * z)) * sp;
    *By += -a2 * cos((double)(k * z2)) * sp;
    *Bz += +a2 * cos((double)(k * z2)) * cp;
  } else {
    const float r = j * L.dy - L.axis, r2 = r + L.dy / 2;
    *Ey += +a * laser_gauss(L, z, r2) * cp;
    *Ez += +a * laser_gauss(L, z, r) * sp;
    *By += -a2 * laser_gauss(L, z2, r) * sp;
    *Bz += +a2 * laser_gauss(L, z2, r2) * cp;
  }
}

// div E = div B = 0 through Ex and Bx, integrated from the right in double,
// one row per thread in the reference's order (div_corr_x, emf.c:213-231)
__global__ void k_laser_divcorr(float *EB, Grid G, float dx, float dy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= G.ny) return;
  const double rxy = dx / dy;
  double ex = 0.0, bx = 0.0;
  const int by = j + 1;
  for (int i = G.nx - 1; i >= 0; --i) {
    const int b = i + 1;
    ex += rxy * (EB[gidx(G, 1, b + 1, by)] - EB[gidx(G, 1, b + 1, by - 1)]);
    EB[gidx(G, 0, b, by)] = ex;
    bx += rxy * (EB[gidx(G, 4, b, by + 1)] - EB[gidx(G, 4, b, by)]);
    EB[gidx(G, 3, b, by)] = bx;
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline dim3 grid_rows(const Grid &G, int bs) { return dim3((G.nx + 3 + bs - 1) / bs, G.ny + 3); }

cudaError_t launch_aos_to_planes(const float *aos, float *planes, const Grid &G, int ncomp, cudaStream_t st) {
  k_aos_to_planes<<<1024, 256, 0, st>>>(aos, planes, G, ncomp);
  return cudaGetLastError();
}

cudaError_t launch_planes_to_aos(const float *planes, float *aos, const Grid &G, int ncomp, cudaStream_t st) {
  k_planes_to_aos<<<1024, 256, 0, st>>>(planes, aos, G, ncomp);
  return cudaGetLastError();
}

cudaError_t launch_fold(float *J, const Grid &G, int mw, cudaStream_t st) {
  if (!mw) k_fold_x<<<(G.ny + 3 + 127) / 128, 128, 0, st>>>(J, G);
  k_fold_y<<<(G.nx + 3 + 127) / 128, 128, 0, st>>>(J, G);
  return cudaGetLastError();
}

// shared memory of one x-filter CTA (a component of a row, double buffered)
size_t smooth_x_smem(const Grid &G) { return sizeof(float) * 2 * (size_t)(G.nx + 3); }

cudaError_t launch_smooth_x_all(float *J, const Grid &G, const SmoothPasses &P, int mw, cudaStream_t st) {
  const size_t sh = smooth_x_smem(G);
  if (sh > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_smooth_x_all, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    if (e != cudaSuccess) return e;
  }
  k_smooth_x_all<<<dim3(G.ny, 3), 256, sh, st>>>(J, G, P, mw);
  return cudaGetLastError();
}

cudaError_t launch_smooth_y_all(const float *Jin, float *Jout, const Grid &G, const SmoothPasses &P,
                                cudaStream_t st) {
  const size_t sh = sizeof(float) * 2 * ((size_t)(kSmoothYRows + 2 * P.n) + 1) * kSmoothYCols;
  dim3 grid((G.nx + 3 + kSmoothYCols - 1) / kSmoothYCols, (G.ny + kSmoothYRows - 1) / kSmoothYRows, 3);
  k_smooth_y_all<<<grid, 256, sh, st>>>(Jin, Jout, G, P);
  return cudaGetLastError();
}

cudaError_t launch_smooth_xy_all(const float *Jin, float *Jout, const Grid &G, const SmoothPasses &PX,
                                 const SmoothPasses &P, int mw, cudaStream_t st) {
  const size_t R = kSmoothYRows + 2 * P.n, XW = kSmoothYCols + 2 * PX.n;
  const size_t sh = sizeof(float) * (2 * R * XW + 2 * kSmoothYCols) + sizeof(int) * R;
  if (sh > 48 * 1024) return cudaErrorInvalidValue;  // more than 8 passes along an axis
  dim3 grid((G.nx + 3 + kSmoothYCols - 1) / kSmoothYCols, (G.ny + kSmoothYRows - 1) / kSmoothYRows, 3);
  k_smooth_xy_all<<<grid, 256, sh, st>>>(Jin, Jout, G, PX, P, mw);
  return cudaGetLastError();
}

cudaError_t launch_yee(const CUtensorMap *tm_eb, const CUtensorMap *tm_j, float *EBout, const Grid &G,
                       const YeeConst &Y, int *err, cudaStream_t st) {
  dim3 grid((G.nx + 3 + kYeeOX - 1) / kYeeOX, (G.ny + 3 + kYeeOY - 1) / kYeeOY);
  k_yee<<<grid, 256, 0, st>>>(*tm_eb, *tm_j, EBout, G, Y, err);
  return cudaGetLastError();
}

cudaError_t launch_emf_gc(float *EB, const Grid &G, int mw, cudaStream_t st) {
  k_emf_gc<<<grid_rows(G, 256), 256, 0, st>>>(EB, G, mw);
  return cudaGetLastError();
}

cudaError_t launch_ext_add(const float *EB, float *EBp, const float *extE, const float *extB, int Etype, int Btype,
                           float3 E0, float3 B0, const Grid &G, cudaStream_t st) {
  k_ext_add<<<grid_rows(G, 256), 256, 0, st>>>(EB, EBp, extE, extB, Etype, Btype, E0, B0, G);
  return cudaGetLastError();
}

cudaError_t launch_window_shift(const float *EBin, float *EBout, const Grid &G, cudaStream_t st) {
  k_window_shift<<<grid_rows(G, 256), 256, 0, st>>>(EBin, EBout, G);
  return cudaGetLastError();
}

cudaError_t launch_emf_energy(const float *EB, const Grid &G, double *partial, int nblocks, double *out, float dx,
                              float dy, cudaStream_t st) {
  k_emf_energy_partial<<<nblocks, 256, 0, st>>>(EB, G, partial);
  k_emf_energy_final<<<1, 32, 0, st>>>(partial, nblocks, out, dx, dy);
  return cudaGetLastError();
}

// one history row: the field energy from the partials (the sum of
// k_emf_energy_final) and the kinetic energy of every species; the row index
// is a device counter, so a captured step appends where it runs
__global__ void k_energy_history_row(const double *partial, int nblocks, float dx, float dy,
                                     double *const *ekin, int nsp, double *hist, int *hist_n, int cap, int cols) {
  const int n = *hist_n;
  __syncthreads();
  if (n >= cap) return;
  double *row = hist + (size_t)n * cols;
  const int t = threadIdx.x;
  if (t < 6) {
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += partial[b * 6 + t];
    row[t] = s * (0.5 * dx * dy);
  } else if (t - 6 < nsp) {
    row[t] = *ekin[t - 6];
  }
  __syncthreads();
  if (t == 0) *hist_n = n + 1;
}

cudaError_t launch_energy_history(const float *EB, const Grid &G, double *partial, int nblocks, double *hist,
                                  int *hist_n, int cap, int cols, double *const *ekin, int nsp, float dx, float dy,
                                  cudaStream_t st) {
  if (nsp + 6 > 64) return cudaErrorInvalidValue;
  k_emf_energy_partial<<<nblocks, 256, 0, st>>>(EB, G, partial);
  k_energy_history_row<<<1, 64, 0, st>>>(partial, nblocks, dx, dy, ekin, nsp, hist, hist_n, cap, cols);
  return cudaGetLastError();
}

__global__ void k_gather_words(int *const *src, int n, int *dst) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = *src[k];
}

cudaError_t launch_gather_words(int *const *src, int n, int *dst, cudaStream_t st) {
  k_gather_words<<<(n + 255) / 256, 256, 0, st>>>(src, n, dst);
  return cudaGetLastError();
}

cudaError_t launch_laser(float *EB, const Grid &G, const LaserConst &L, cudaStream_t st) {
  dim3 grid((G.nx + 127) / 128, G.ny);
  k_laser_fields<<<grid, 128, 0, st>>>(EB, G, L);
  if (L.type == 1) k_laser_divcorr<<<(G.ny + 63) / 64, 64, 0, st>>>(EB, G, L.dx, L.dy);
  return cudaGetLastError();
}

}  // namespace zc
