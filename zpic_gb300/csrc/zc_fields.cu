// zc_fields.cu -- grid kernels of libzpic_cuda (sm_103a): current guard-cell
// fold and digital filtering, the fused Yee field advance, field guard
// cells, external fields, moving window, laser launch and FP64 energies.
//
// Compiled with -fmad=false: every cell is computed with the same float32
// operations, in the same order, as the reference (em2d/current.c,
// em2d/emf.c), so from the same inputs these kernels return the same bits.
// All of them are HBM-bound stencils; none is a contraction.
#include <math.h>

#include <type_traits>

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
  // one thread per (buffer row, component), in the reference's order: cells
  // -1, 0, 1 add nx-1, nx, nx+1, then those take the sums (the order matters
  // when the pairs overlap, nx < 3)
  const int n = (G.ny + 3) * 3;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    const int by = g / 3, c = g % 3;
#pragma unroll
    for (int b = 0; b < 3; ++b) J[gidx(G, c, b, by)] += J[gidx(G, c, G.nx + b, by)];
#pragma unroll
    for (int b = 0; b < 3; ++b) J[gidx(G, c, G.nx + b, by)] = J[gidx(G, c, b, by)];
  }
}

__global__ void k_fold_y(float *J, Grid G) {
  // one thread per (buffer column, component), in the reference's order
  const int gx = G.nx + 3, n = gx * 3;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    const int bx = g % gx, c = g / gx;
#pragma unroll
    for (int b = 0; b < 3; ++b) J[gidx(G, c, bx, b)] += J[gidx(G, c, bx, G.ny + b)];
#pragma unroll
    for (int b = 0; b < 3; ++b) J[gidx(G, c, bx, G.ny + b)] = J[gidx(G, c, bx, b)];
  }
}

// Both folds in one launch (periodic x): the x pairs of the rows outside the
// y guard bands, the y pairs of the columns outside the x guard bands, and
// every corner quad as the two folds leave it, (J(b,b') + J(nx+b,b')) +
// (J(b,ny+b') + J(nx+b,ny+b')) in all four cells: the same float additions
// as k_fold_x followed by k_fold_y.  Needs nx, ny >= 6 (disjoint bands).
__global__ void k_fold_xy(float *J, Grid G) {
  const int nx = G.nx, ny = G.ny;
  const int nA = (ny - 3) * 9, nB = (nx - 3) * 9, n = nA + nB + 27;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    if (g < nA) {  // row 3 .. ny - 1: x pair b
      const int by = 3 + g / 9, c = (g % 9) / 3, b = g % 3;
      const size_t lo = gidx(G, c, b, by), hi = gidx(G, c, nx + b, by);
      const float v = J[lo] + J[hi];
      J[lo] = v;
      J[hi] = v;
    } else if (g < nA + nB) {  // column 3 .. nx - 1: y pair b
      const int h = g - nA, bx = 3 + h / 9, c = (h % 9) / 3, b = h % 3;
      const size_t lo = gidx(G, c, bx, b), hi = gidx(G, c, bx, ny + b);
      const float v = J[lo] + J[hi];
      J[lo] = v;
      J[hi] = v;
    } else {  // corner quad (b, b')
      const int h = g - nA - nB, c = h / 9, b = (h % 9) / 3, bp = h % 3;
      const size_t a00 = gidx(G, c, b, bp), a10 = gidx(G, c, nx + b, bp);
      const size_t a01 = gidx(G, c, b, ny + bp), a11 = gidx(G, c, nx + b, ny + bp);
      const float lo = J[a00] + J[a10], hi = J[a01] + J[a11];
      const float v = lo + hi;
      J[a00] = v;
      J[a10] = v;
      J[a01] = v;
      J[a11] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// one [sa, sb, sa] filter tap (kernel_x / kernel_y, em2d/current.c:316-413)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float f3pt(float sa, float sb, float l, float m, float u) {
  return sa * l + sb * m + sa * u;
}

// ---------------------------------------------------------------------------
// All filter passes, along x and then along y, in one sweep over J and
// without shared memory.  A warp owns 32 consecutive buffer columns -- HX
// halo columns on each side (periodic images of interior columns, or with a
// moving window the columns themselves, zero outside the buffer), so that it
// writes W = 32 - 2 HX of them -- and walks down a block of rows plus H halo
// rows above and below (periodic over the interior rows).  Each row is read
// once and filtered along x by HX passes across the lanes (kernel_x; after
// p passes lanes p .. 31-p hold filtered values; a moving window's guard
// columns stay as they are).  The rows then go through H y-pass stages held
// in registers (kernel_y): stage p keeps the last two rows it received and,
// given the next one, emits the filtered middle row to stage p + 1, so the
// last stage emits rows H behind the walk.  Only interior columns are
// filtered along y, and the first y pass reads the y guard rows as stored
// (the x passes leave them untouched).  The y guard rows of the result are
// periodic copies of the filtered rows, or, without y passes, the rows as
// stored.  Every cell sees the same float operations in the same order as
// with one kernel per pass (em2d/current.c:316-413).
// ---------------------------------------------------------------------------
constexpr int kSmoothRows = 32;  // interior rows per warp
constexpr int kSmoothRing = 16;  // rows in flight per warp (asynchronous copies)
constexpr int kSmoothWarps = 8;  // warps per CTA

// NX, NY: the pass counts when known at compile time (exact loops, no
// branches per row), or -1 to read them from PX, PY (up to kMaxSmoothPasses)
template <int NX, int NY>
__global__ void __launch_bounds__(32 * kSmoothWarps) k_smooth(const float *Jin, float *Jout, Grid G, SmoothPasses PX,
                                                              SmoothPasses PY, int mw) {
  constexpr int MX = NX >= 0 ? NX : kMaxSmoothPasses;  // loop bounds
  constexpr int MY = NY >= 0 ? NY : kMaxSmoothPasses;
  // each warp streams its rows through a private ring of row slots: a lane
  // copies and later reads only its own column, so no synchronisation is
  // needed beyond the copies' own completion
  __shared__ float ring[kSmoothWarps][kSmoothRing][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int HX = NX >= 0 ? NX : PX.n, H = NY >= 0 ? NY : PY.n;
  const int W = 32 - 2 * HX;
  const int gx = G.nx + 3;
  const int nstrip = (gx + W - 1) / W;
  const int nblk = (G.ny + kSmoothRows - 1) / kSmoothRows;
  const int wid = blockIdx.x * kSmoothWarps + w;
  if (wid >= nstrip * nblk) return;  // whole warps leave together
  const int c = blockIdx.y;
  const int strip = wid % nstrip, blk = wid / nstrip;
  const int b = strip * W - HX + lane;  // this lane's buffer column
  int src = b;
  bool have = true;
  if (mw) have = b >= 0 && b < gx;
  else if (b < 1 || b > G.nx) src = ((b - 1) % G.nx + G.nx) % G.nx + 1;
  const bool xfilt = (lane > 0 && lane < 31) && (!mw || (b >= 1 && b <= G.nx));
  const bool yfilt = b >= 1 && b <= G.nx;
  const bool writer = lane >= HX && lane < 32 - HX && b < gx;
  const float *col = Jin + c * G.plane + (have ? src : 0);
  float *out = Jout + c * G.plane + b;
  const int j0 = blk * kSmoothRows;
  const int nrows = min(kSmoothRows, G.ny - j0);
  const int R = nrows + 2 * H;  // rows walked
  float *slot = &ring[w][0][lane];
  int jw = (j0 - H) % G.ny;  // interior row of walk row 0
  if (jw < 0) jw += G.ny;
  // the first kSmoothRing rows in flight, one copy group per row
  int jl = jw;  // interior row of the next row to copy
#pragma unroll 1
  for (int d = 0; d < kSmoothRing; ++d) {
    if (d < R) cp_async4_zfill(slot + d * 32, have ? col + (size_t)(jl + 1) * G.pitch : Jin, have);
    cp_async_commit();
    jl = (jl + 1 == G.ny) ? 0 : jl + 1;
  }
  const float glo = have ? col[0] : 0.f;                             // guard row -1 as stored
  const float ghi = have ? col[(size_t)(G.ny + 1) * G.pitch] : 0.f;  // guard row ny as stored
  if (H == 0 && blk == 0 && writer) {
    // without y passes the y guard rows keep their values
    out[0] = glo;
    out[(size_t)(G.ny + 1) * G.pitch] = ghi;
    out[(size_t)(G.ny + 2) * G.pitch] = have ? col[(size_t)(G.ny + 2) * G.pitch] : 0.f;
  }
  float s0[MY > 0 ? MY : 1], s1[MY > 0 ? MY : 1];  // each stage's last two rows
  int jprev = (jw == 0) ? G.ny - 1 : jw - 1;      // interior row of walk row rr - 1

  // one walk row; FILL: the first 2H rows, while the stages fill up
  auto step = [&](int rr, auto fill) {
    constexpr bool FILL = decltype(fill)::value;
    cp_async_wait<kSmoothRing - 1>();  // row rr has arrived
    const int k = rr & (kSmoothRing - 1);
    float v = slot[k * 32];
    // the slot is free again: copy row rr + kSmoothRing into it
    if (rr + kSmoothRing < R) cp_async4_zfill(slot + k * 32, have ? col + (size_t)(jl + 1) * G.pitch : Jin, have);
    cp_async_commit();
    jl = (jl + 1 == G.ny) ? 0 : jl + 1;
#pragma unroll
    for (int p = 0; p < MX; ++p) {
      if (NX < 0 && p >= HX) break;
      const float l = __shfl_up_sync(0xffffffffu, v, 1);
      const float u = __shfl_down_sync(0xffffffffu, v, 1);
      if (xfilt) v = f3pt(PX.sa[p], PX.sb[p], l, v, u);
    }
    // stage p receives walk row rr - p (stage p - 1 emits rows p .. on) and
    // emits the middle row once it holds the two rows below
    bool emit = true;
#pragma unroll
    for (int p = 0; p < MY; ++p) {
      if (NY < 0 && p >= H) break;
      const bool ready = !FILL || rr - p >= p + 2;
      float e = 0.f;
      if (ready) {
        float lo = s0[p], hi = v;
        if (p == 0) {
          // the middle row next to a y guard row reads it as stored
          lo = (jprev == 0) ? glo : lo;
          hi = (jprev == G.ny - 1) ? ghi : hi;
        }
        e = yfilt ? f3pt(PY.sa[p], PY.sb[p], lo, s1[p], hi) : s1[p];
      }
      s0[p] = s1[p];
      s1[p] = v;
      if (FILL && !ready) {
        emit = false;
        break;
      }
      v = e;
    }
    jprev = (jprev + 1 == G.ny) ? 0 : jprev + 1;
    // the last stage emits walk row rr - H; rows H .. R-1-H are the output
    if ((!FILL || (emit && rr >= 2 * H)) && writer) {
      const int j = j0 + rr - 2 * H;
      out[(size_t)(j + 1) * G.pitch] = v;
      if (H > 0) {
        if (j == G.ny - 1) out[0] = v;
        if (j < 2) out[(size_t)(G.ny + 1 + j) * G.pitch] = v;
      }
    }
  };
  const int nfill = min(2 * H, R);
#pragma unroll 1
  for (int rr = 0; rr < nfill; ++rr) step(rr, std::true_type{});
#pragma unroll 2
  for (int rr = nfill; rr < R; ++rr) step(rr, std::false_type{});
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// The same filter for up to 4 passes per axis, four columns per lane: a
// warp owns 128 consecutive buffer columns (the first and last lane hold
// halo columns only), so it writes 120 of them, moves its rows with 16-byte
// copies where a lane's four columns are stored side by side (periodic
// images and columns outside a moving window's buffer are copied one by
// one) and filters four columns per instruction.  Every cell sees the
// same float operations in the same order as k_smooth (and as one kernel
// per pass, em2d/current.c:316-413).
// ---------------------------------------------------------------------------
#ifndef ZC_S4_ROWS
#define ZC_S4_ROWS 32
#endif
#ifndef ZC_S4_RING
#define ZC_S4_RING 8
#endif
#ifndef ZC_S4_WARPS
#define ZC_S4_WARPS 8
#endif
constexpr int kS4Rows = ZC_S4_ROWS;    // interior rows per warp
constexpr int kS4Ring = ZC_S4_RING;    // rows in flight per warp (a power of two)
constexpr int kS4Warps = ZC_S4_WARPS;  // warps per CTA
constexpr int kS4W = 120;    // columns a warp writes

#ifndef ZC_S4_MINB
#define ZC_S4_MINB 3
#endif

// four columns; with SEL the columns whose `on` is false keep m
// (scalar float32 operations: packed pair products and sums were measured
// to round differently from the scalar ones once a product and a sum follow
// each other, so the bit-exact filter keeps the scalar form)
template <bool SEL>
__device__ __forceinline__ float4 f3pt4(float sa, float sb, const float4 &l, const float4 &m, const float4 &u,
                                        const bool (&on)[4]) {
  float4 r = make_float4(f3pt(sa, sb, l.x, m.x, u.x), f3pt(sa, sb, l.y, m.y, u.y), f3pt(sa, sb, l.z, m.z, u.z),
                         f3pt(sa, sb, l.w, m.w, u.w));
  if (SEL) {
    r.x = on[0] ? r.x : m.x;
    r.y = on[1] ? r.y : m.y;
    r.z = on[2] ? r.z : m.z;
    r.w = on[3] ? r.w : m.w;
  }
  return r;
}

template <int NX, int NY>
__global__ void __launch_bounds__(32 * kS4Warps, ZC_S4_MINB) k_smooth4(const float *Jin, float *Jout, Grid G, SmoothPasses PX,
                                                           SmoothPasses PY, int mw) {
  __shared__ __align__(16) float4 ring[kS4Warps][kS4Ring][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gx = G.nx + 3;
  const int nstrip = (gx + kS4W - 1) / kS4W;
  const int nblk = (G.ny + kS4Rows - 1) / kS4Rows;
  const int wid = blockIdx.x * kS4Warps + w;
  if (wid >= nstrip * nblk) return;  // whole warps leave together
  const int c = blockIdx.y;
  const int strip = wid % nstrip, blk = wid / nstrip;
  const int b0 = strip * kS4W - 4 + 4 * lane;  // this lane's first buffer column
  // per column: source column (periodic image), presence, x and y filtering
  int src[4];
  bool have[4], xf[4], yf[4];
  bool direct = true;  // four present columns stored side by side: one 16-byte copy
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int b = b0 + e, q = 4 * lane + e;
    src[e] = b;
    have[e] = true;
    if (mw) have[e] = b >= 0 && b < gx;
    else if (b < 1 || b > G.nx) src[e] = ((b - 1) % G.nx + G.nx) % G.nx + 1;
    xf[e] = (q >= 1 && q <= 126) && (!mw || (b >= 1 && b <= G.nx));
    yf[e] = b >= 1 && b <= G.nx;
    direct = direct && have[e] && src[e] == b;
  }
  // Warp-uniform: whether any column must keep its value in an x or a y
  // pass.  The warp's outer columns (q = 0 and 127) do not count for x:
  // filtered with a wrong neighbour, their error moves one column inward per
  // pass and reaches at most column 3 after 4 passes, and columns 0..3 and
  // 124..127 are never written.
  bool xkeep = false, ykeep = false;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int q = 4 * lane + e;
    xkeep = xkeep || (!xf[e] && q >= 1 && q <= 126);
    ykeep = ykeep || !yf[e];
  }
  const bool xsel = __any_sync(0xffffffffu, xkeep), ysel = __any_sync(0xffffffffu, ykeep);
  const bool writer = lane >= 1 && lane <= 30;
  const float *pin = Jin + c * G.plane;
  float *out = Jout + c * G.plane;
  const int j0 = blk * kS4Rows;
  const int nrows = min(kS4Rows, G.ny - j0);
  const int R = nrows + 2 * NY;  // rows walked
  float4 *slot = &ring[w][0][lane];
  int jw = (j0 - NY) % G.ny;  // interior row of walk row 0
  if (jw < 0) jw += G.ny;
  auto copy_row = [&](float4 *dst, int jrow) {  // buffer row jrow + 1
    const float *r = pin + (size_t)(jrow + 1) * G.pitch;
    if (direct) {
      cp_async16(dst, r + b0);
    } else {
      float *d = reinterpret_cast<float *>(dst);
#pragma unroll
      for (int e = 0; e < 4; ++e) cp_async4_zfill(d + e, have[e] ? r + src[e] : Jin, have[e]);
    }
  };
  int jl = jw;  // interior row of the next row to copy
#pragma unroll 1
  for (int d = 0; d < kS4Ring; ++d) {
    if (d < R) copy_row(slot + d * 32, jl);
    cp_async_commit();
    jl = (jl + 1 == G.ny) ? 0 : jl + 1;
  }
  float4 glo, ghi;  // guard rows -1 and ny as stored
  {
    float lo[4], hi[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      lo[e] = have[e] ? pin[src[e]] : 0.f;
      hi[e] = have[e] ? pin[(size_t)(G.ny + 1) * G.pitch + src[e]] : 0.f;
    }
    glo = make_float4(lo[0], lo[1], lo[2], lo[3]);
    ghi = make_float4(hi[0], hi[1], hi[2], hi[3]);
  }
  // writes four columns of one output buffer row (the last strip may end
  // past the buffer)
  auto put = [&](int brow, const float4 &v) {
    float *o = out + (size_t)brow * G.pitch + b0;
    if (b0 + 3 < gx) {
      *reinterpret_cast<float4 *>(o) = v;
    } else {
      const float a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (b0 + e < gx) o[e] = a[e];
    }
  };
  if (NY == 0 && blk == 0 && writer) {
    // without y passes the y guard rows keep their values
    put(0, glo);
    put(G.ny + 1, ghi);
    float t[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) t[e] = have[e] ? pin[(size_t)(G.ny + 2) * G.pitch + src[e]] : 0.f;
    put(G.ny + 2, make_float4(t[0], t[1], t[2], t[3]));
  }
  float4 s0[NY > 0 ? NY : 1], s1[NY > 0 ? NY : 1];  // each stage's last two rows
  int jprev = (jw == 0) ? G.ny - 1 : jw - 1;       // interior row of walk row rr - 1

  auto step = [&](int rr, auto fill) {
    constexpr bool FILL = decltype(fill)::value;
    cp_async_wait<kS4Ring - 1>();  // row rr has arrived
    const int k = rr & (kS4Ring - 1);
    float4 v = slot[k * 32];
    // the slot is free again: copy row rr + kS4Ring into it
    if (rr + kS4Ring < R) copy_row(slot + k * 32, jl);
    cp_async_commit();
    jl = (jl + 1 == G.ny) ? 0 : jl + 1;
#pragma unroll
    for (int p = 0; p < NX; ++p) {
      const float l = __shfl_up_sync(0xffffffffu, v.w, 1);
      const float u = __shfl_down_sync(0xffffffffu, v.x, 1);
      const float4 lv = make_float4(l, v.x, v.y, v.z), uv = make_float4(v.y, v.z, v.w, u);
      v = xsel ? f3pt4<true>(PX.sa[p], PX.sb[p], lv, v, uv, xf) : f3pt4<false>(PX.sa[p], PX.sb[p], lv, v, uv, xf);
    }
    // stage p receives walk row rr - p and emits the middle row once it
    // holds the two rows below
    bool emit = true;
#pragma unroll
    for (int p = 0; p < NY; ++p) {
      const bool ready = !FILL || rr - p >= p + 2;
      float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ready) {
        float4 lo = s0[p], hi = v;
        if (p == 0) {
          // the middle row next to a y guard row reads it as stored
          lo = (jprev == 0) ? glo : lo;
          hi = (jprev == G.ny - 1) ? ghi : hi;
        }
        e = ysel ? f3pt4<true>(PY.sa[p], PY.sb[p], lo, s1[p], hi, yf)
                 : f3pt4<false>(PY.sa[p], PY.sb[p], lo, s1[p], hi, yf);
      }
      s0[p] = s1[p];
      s1[p] = v;
      if (FILL && !ready) {
        emit = false;
        break;
      }
      v = e;
    }
    jprev = (jprev + 1 == G.ny) ? 0 : jprev + 1;
    // the last stage emits walk row rr - NY; rows NY .. R-1-NY are the output
    if ((!FILL || (emit && rr >= 2 * NY)) && writer) {
      const int j = j0 + rr - 2 * NY;
      put(j + 1, v);
      if (NY > 0) {
        if (j == G.ny - 1) put(0, v);
        if (j < 2) put(G.ny + 1 + j, v);
      }
    }
  };
  const int nfill = min(2 * NY, R);
#pragma unroll 1
  for (int rr = 0; rr < nfill; ++rr) step(rr, std::true_type{});
#pragma unroll 2
  for (int rr = nfill; rr < R; ++rr) step(rr, std::false_type{});
  cp_async_wait<0>();
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
// a value stored at (bx, by) and at its periodic guard images (xm, ym; -1: none)
__device__ __forceinline__ void put_mirrored(float *EB, const Grid &G, int c, int bx, int by, int xm, int ym,
                                             float v) {
  EB[gidx(G, c, bx, by)] = v;
  if (xm >= 0) EB[gidx(G, c, xm, by)] = v;
  if (ym >= 0) EB[gidx(G, c, bx, ym)] = v;
  if (xm >= 0 && ym >= 0) EB[gidx(G, c, xm, ym)] = v;
}

#ifndef ZC_YEE_MINB
#define ZC_YEE_MINB 6
#endif
__global__ void __launch_bounds__(256, ZC_YEE_MINB) k_yee(const __grid_constant__ CUtensorMap tm_eb,
                                             const __grid_constant__ CUtensorMap tm_j, float *EBout, Grid G,
                                             YeeConst Y, int *err, double *epart, float *jzero, int gc) {
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
  // B2 on the output tile, then store E1 and B2; with epart, the squares of
  // the interior cells' new values are summed for the field energy
  float se[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
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
    if (jzero) {  // the raw deposit buffer, dead once filtered: cleared for the next step
      jzero[gidx(G, 0, bx, by)] = 0.f;
      jzero[gidx(G, 1, bx, by)] = 0.f;
      jzero[gidx(G, 2, bx, by)] = 0.f;
    }
    if (gc) {
      // guard cells as emf_update_gc leaves them (emf.c:573-637): a guard
      // cell is not stored here; the cell it copies stores its value there
      // too (periodic in x unless the window moves, always in y)
      const bool gxc = !Y.mw && (bx == 0 || bx > nx), gyc = (by == 0 || by > ny);
      if (gxc || gyc) continue;
      const int xm = Y.mw ? -1 : (bx == nx ? 0 : (bx <= 2 ? nx + bx : -1));
      const int ym = by == ny ? 0 : (by <= 2 ? ny + by : -1);
      put_mirrored(EBout, G, 0, bx, by, xm, ym, Ex[s]);
      put_mirrored(EBout, G, 1, bx, by, xm, ym, Ey[s]);
      put_mirrored(EBout, G, 2, bx, by, xm, ym, Ez[s]);
      put_mirrored(EBout, G, 3, bx, by, xm, ym, bxv);
      put_mirrored(EBout, G, 4, bx, by, xm, ym, byv);
      put_mirrored(EBout, G, 5, bx, by, xm, ym, bzv);
    } else {
      EBout[gidx(G, 0, bx, by)] = Ex[s];
      EBout[gidx(G, 1, bx, by)] = Ey[s];
      EBout[gidx(G, 2, bx, by)] = Ez[s];
      EBout[gidx(G, 3, bx, by)] = bxv;
      EBout[gidx(G, 4, bx, by)] = byv;
      EBout[gidx(G, 5, bx, by)] = bzv;
    }
    if (epart && bx >= 1 && bx <= nx && by >= 1 && by <= ny) {
      se[0] += Ex[s] * Ex[s];
      se[1] += Ey[s] * Ey[s];
      se[2] += Ez[s] * Ez[s];
      se[3] += bxv * bxv;
      se[4] += byv * byv;
      se[5] += bzv * bzv;
    }
  }
  if (epart) {
    // warp sums in float (64 cells a warp), then doubles across the warps
    __shared__ double swe[6][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      float v = se[c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) swe[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
      double v = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) v += swe[threadIdx.x][w];
      epart[(blockIdx.y * gridDim.x + blockIdx.x) * 6 + threadIdx.x] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// periodic guard cells of E and B (emf_update_gc, em2d/emf.c:573-637): x
// unless the window moves, y always.  Guards only read interior rows.
// ---------------------------------------------------------------------------
__global__ void k_emf_gc(float *EB, Grid G, int mw) {
  // one thread per guard cell: buffer columns 0, nx+1, nx+2 of every row
  // (not under a moving window), then buffer rows 0, ny+1, ny+2 of every
  // column (the corners come up twice and get the same value)
  const int gx = G.nx + 3, gy = G.ny + 3;
  const int ncol = mw ? 0 : 3 * gy, n = ncol + 3 * gx;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    int bx, by;
    if (g < ncol) {
      const int b = g % 3;
      by = g / 3;
      bx = b ? G.nx + b : 0;
    } else {
      const int h = g - ncol, b = h / gx;
      bx = h % gx;
      by = b ? G.ny + b : 0;
    }
    const bool gxg = (bx == 0 || bx > G.nx), gyg = (by == 0 || by > G.ny);
    int sx = bx, sy = by;
    if (gxg && !mw) sx = (bx == 0) ? G.nx : bx - G.nx;
    if (gyg) sy = (by == 0) ? G.ny : by - G.ny;
    if (sx == bx && sy == by) continue;
    for (int c = 0; c < 6; ++c) EB[gidx(G, c, bx, by)] = EB[gidx(G, c, sx, sy)];
  }
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
  // the 32 lanes' sums (s - cc each) as float pairs added with the exact
  // two-sum (hi + lo carries about 48 bits), then one double per warp: the
  // float pipes do the tree, FP64 (a slow pipe on this part) only the last
  // eight additions of a block
  __shared__ double swarp[6][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    float hi = s[c], lo = -cc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
      const float t = hi + oh, bb = t - hi;
      const float e = (hi - (t - bb)) + (oh - bb);
      hi = t;
      lo = lo + ol + e;
    }
    if (lane == 0) swarp[c][warp] = (double)hi + (double)lo;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) v += swarp[threadIdx.x][w];
    partial[blockIdx.x * 6 + threadIdx.x] = v;
  }
}

// the sum over the blocks of component c of the partials, by warp c (lanes
// take every 32nd block, then a shuffle tree): valid in lane 0
__device__ __forceinline__ double partial_sum(const double *partial, int nblocks, int c) {
  // four running sums a lane, so that four loads are in flight
  const int lane = threadIdx.x & 31;
  double a[4] = {0, 0, 0, 0};
  for (int b = lane; b < nblocks; b += 128) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (b + 32 * u < nblocks) a[u] += partial[(b + 32 * u) * 6 + c];
  }
  double s = (a[0] + a[1]) + (a[2] + a[3]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return s;
}

// six warps, one per component
__global__ void k_emf_energy_final(const double *partial, int nblocks, double *out, float dx, float dy) {
  const int c = threadIdx.x >> 5;
  if (c >= 6) return;
  const double s = partial_sum(partial, nblocks, c);
  if ((threadIdx.x & 31) == 0) out[c] = s * (0.5 * dx * dy);
}

// ---------------------------------------------------------------------------
// laser launch (emf_add_laser, em2d/emf.c:158-350): same double-precision
// library calls on float arguments as the reference
// ---------------------------------------------------------------------------
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
  if (!mw && G.nx >= 6 && G.ny >= 6) {
    k_fold_xy<<<((G.nx + G.ny - 6) * 9 + 27 + 255) / 256, 256, 0, st>>>(J, G);
    return cudaGetLastError();
  }
  if (!mw) k_fold_x<<<((G.ny + 3) * 3 + 255) / 256, 256, 0, st>>>(J, G);
  k_fold_y<<<((G.nx + 3) * 3 + 255) / 256, 256, 0, st>>>(J, G);
  return cudaGetLastError();
}

cudaError_t launch_smooth(const float *Jin, float *Jout, const Grid &G, const SmoothPasses &PX,
                          const SmoothPasses &PY, int mw, cudaStream_t st) {
  if (PX.n > kMaxSmoothPasses || PY.n > kMaxSmoothPasses || PX.n > 15) return cudaErrorInvalidValue;
  if (PX.n <= 4 && PY.n <= 4) {
    // four columns per lane
    const long long warps4 = (long long)((G.nx + 3 + kS4W - 1) / kS4W) * ((G.ny + kS4Rows - 1) / kS4Rows);
    const dim3 grid4((unsigned)((warps4 + kS4Warps - 1) / kS4Warps), 3);
#define ZC_SMOOTH4(A, B)                                                          \
    if (PX.n == A && PY.n == B) {                                                 \
      k_smooth4<A, B><<<grid4, 32 * kS4Warps, 0, st>>>(Jin, Jout, G, PX, PY, mw); \
      return cudaGetLastError();                                                  \
    }
#define ZC_SMOOTH4_ROW(A) ZC_SMOOTH4(A, 0) ZC_SMOOTH4(A, 1) ZC_SMOOTH4(A, 2) ZC_SMOOTH4(A, 3) ZC_SMOOTH4(A, 4)
    ZC_SMOOTH4_ROW(0)
    ZC_SMOOTH4_ROW(1)
    ZC_SMOOTH4_ROW(2)
    ZC_SMOOTH4_ROW(3)
    ZC_SMOOTH4_ROW(4)
#undef ZC_SMOOTH4_ROW
#undef ZC_SMOOTH4
  }
  const int W = 32 - 2 * PX.n;
  const long long warps = (long long)((G.nx + 3 + W - 1) / W) * ((G.ny + kSmoothRows - 1) / kSmoothRows);
  const dim3 grid((unsigned)((warps + kSmoothWarps - 1) / kSmoothWarps), 3);
  const int block = 32 * kSmoothWarps;
  // exact pass counts for up to 4 passes per axis, else counts read at run time
#define ZC_SMOOTH(A, B)                                                     \
  if (PX.n == A && PY.n == B) {                                            \
    k_smooth<A, B><<<grid, block, 0, st>>>(Jin, Jout, G, PX, PY, mw);      \
    return cudaGetLastError();                                             \
  }
#define ZC_SMOOTH_ROW(A) ZC_SMOOTH(A, 0) ZC_SMOOTH(A, 1) ZC_SMOOTH(A, 2) ZC_SMOOTH(A, 3) ZC_SMOOTH(A, 4)
  ZC_SMOOTH_ROW(0)
  ZC_SMOOTH_ROW(1)
  ZC_SMOOTH_ROW(2)
  ZC_SMOOTH_ROW(3)
  ZC_SMOOTH_ROW(4)
#undef ZC_SMOOTH_ROW
#undef ZC_SMOOTH
  k_smooth<-1, -1><<<grid, block, 0, st>>>(Jin, Jout, G, PX, PY, mw);
  return cudaGetLastError();
}

int yee_blocks(const Grid &G) { return ((G.nx + 3 + kYeeOX - 1) / kYeeOX) * ((G.ny + 3 + kYeeOY - 1) / kYeeOY); }

cudaError_t launch_yee(const CUtensorMap *tm_eb, const CUtensorMap *tm_j, float *EBout, const Grid &G,
                       const YeeConst &Y, int *err, double *epart, float *jzero, bool gc, cudaStream_t st) {
  if (gc && (G.nx < 3 || G.ny < 3)) return cudaErrorInvalidValue;  // mirrors would overlap
  dim3 grid((G.nx + 3 + kYeeOX - 1) / kYeeOX, (G.ny + 3 + kYeeOY - 1) / kYeeOY);
  k_yee<<<grid, 256, 0, st>>>(*tm_eb, *tm_j, EBout, G, Y, err, epart, jzero, gc ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_emf_gc(float *EB, const Grid &G, int mw, cudaStream_t st) {
  k_emf_gc<<<(3 * (G.nx + 3) + 3 * (G.ny + 3) + 255) / 256, 256, 0, st>>>(EB, G, mw);
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
  k_emf_energy_final<<<1, 6 * 32, 0, st>>>(partial, nblocks, out, dx, dy);
  return cudaGetLastError();
}

// the field energy from the partials and the kinetic energy of every
// species, written straight to the caller's (page-locked, mapped) host arrays
__global__ void k_energy_direct(const double *partial, int nblocks, float dx, float dy, EkinRefs K, int nsp,
                                double *emf, double *kin) {
  const int t = threadIdx.x, c = t >> 5;
  if (c < 6) {
    if (emf) {  // (the same for every lane of the warp)
      const double s = partial_sum(partial, nblocks, c);
      if ((t & 31) == 0) emf[c] = s * (0.5 * dx * dy);
    }
  } else if (t - 6 * 32 < nsp && kin) {
    kin[t - 6 * 32] = *K.p[t - 6 * 32];
  }
}

// one history row: the field energy from the partials (the sum of
// k_emf_energy_final) and the kinetic energy of every species; the row index
// is a device counter, so a captured step appends where it runs
__global__ void __launch_bounds__(256) k_energy_history_row(const double *partial, int nblocks, float dx, float dy,
                                                            double *const *ekin, const KinSum *ks, int nsp,
                                                            double *hist, int *hist_n, int cap, int cols) {
  __shared__ double sred[8];
  const int t = threadIdx.x, c = t >> 5, lane = t & 31;
  if (ks) {
    // each species' kinetic energy from its tile partials, by the whole
    // block (as k_sum_energy would leave it in *ekin), before the row
    for (int k = 0; k < nsp; ++k) {
      const KinSum &K = ks[k];
      double s = 0;
      for (int i = t; i < K.ntiles; i += 256) s += K.tiles[i];
      s = block_sum_double<256>(s, sred);
      if (t == 0) {
        if (K.det) {
          const long long *w = reinterpret_cast<const long long *>(K.extra);
          s += efix_join(w[0], w[1]);
        } else {
          s += *K.extra;
        }
        *ekin[k] = K.q_mq * s * dx * dy;  // spec->energy (particles.c:1231)
      }
    }
  }
  __syncthreads();
  const int n = *hist_n;
  __syncthreads();
  if (n >= cap) return;
  double *row = hist + (size_t)n * cols;
  if (c < 6) {  // warps 0..5: the field components
    const double s = partial_sum(partial, nblocks, c);
    if (lane == 0) row[c] = s * (0.5 * dx * dy);
  } else if (t - 6 * 32 < nsp) {  // then one thread per species
    row[6 + t - 6 * 32] = *ekin[t - 6 * 32];
  }
  __syncthreads();
  if (t == 0) *hist_n = n + 1;
}

cudaError_t launch_energy_direct(const float *EB, const Grid &G, double *partial, int nblocks, float dx, float dy,
                                 const EkinRefs &K, int nsp, double *emf, double *kin, cudaStream_t st) {
  if (nsp > kEkinRefs) return cudaErrorInvalidValue;
  if (emf) k_emf_energy_partial<<<nblocks, 256, 0, st>>>(EB, G, partial);
  k_energy_direct<<<1, 6 * 32 + kEkinRefs, 0, st>>>(partial, nblocks, dx, dy, K, nsp, emf, kin);
  return cudaGetLastError();
}

cudaError_t launch_energy_history(const float *EB, const Grid &G, double *partial, int nblocks, double *hist,
                                  int *hist_n, int cap, int cols, double *const *ekin, const KinSum *ks, int nsp,
                                  float dx, float dy, cudaStream_t st) {
  if (nsp > 64) return cudaErrorInvalidValue;
  if (EB) k_emf_energy_partial<<<nblocks, 256, 0, st>>>(EB, G, partial);  // (no EB: partials already made)
  k_energy_history_row<<<1, 256, 0, st>>>(partial, nblocks, dx, dy, ekin, ks, nsp, hist, hist_n, cap, cols);
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
