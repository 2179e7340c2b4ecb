// zc_particles.cu -- particle kernels of libzpic_cuda (sm_103a).
//
// Compiled with -fmad=false: the per-particle arithmetic rounds operation by
// operation exactly like the reference C (em2d/particles.c), so a particle
// advanced here from the same fields lands on the same bits.
//
//   k_push_tiles    one CTA per particle tile: TMA-stages the tile's E/B halo
//                   into shared memory, pushes every particle of the tile
//                   (staggered bilinear gather + relativistic Boris + zigzag
//                   charge-conserving deposit into a shared-memory J tile),
//                   compacts the particles that stay, posts the ones that
//                   leave to the tile's outbox, then adds the J tile into
//                   global J with one TMA reduce-add.
//   k_push_spill    the same physics for particles that did not fit a tile
//                   (global-memory gather and atomics; normally empty).
//   k_migrate       one CTA per tile: pulls the particles bound for it out of
//                   the outboxes of its (up to 8) neighbours.
//   re-layout       upload, moving-window injection and capacity changes.
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc {

// ---------------------------------------------------------------------------
// field / current accessors: shared-memory tile (with a 1-cell lower halo)
// or the global padded planes
// ---------------------------------------------------------------------------
template <int BW, int PL>
struct TileFields {
  const float *s;
  __device__ __forceinline__ float operator()(int c, int i, int j) const {
    return s[c * PL + (j + 1) * BW + (i + 1)];
  }
};
template <int BW, int PL>
struct TileCurrent {
  float *s;
  __device__ __forceinline__ void add(int c, int i, int j, float v) const {
    atomicAdd(&s[c * PL + (j + 1) * BW + (i + 1)], v);
  }
};
struct GlobalFields {
  const float *g;
  int pitch;
  size_t plane;
  __device__ __forceinline__ float operator()(int c, int i, int j) const {
    return __ldg(&g[c * plane + (size_t)(j + 1) * pitch + (i + 1)]);
  }
};
struct GlobalCurrent {
  float *g;
  int pitch;
  size_t plane;
  __device__ __forceinline__ void add(int c, int i, int j, float v) const {
    atomicAdd(&g[c * plane + (size_t)(j + 1) * pitch + (i + 1)], v);
  }
};

// ---------------------------------------------------------------------------
// per-particle physics (restates em2d/particles.c:1029-1226)
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ float lerp2(const F &f, int c, int a, int b, float wa, float wb) {
  return (f(c, a, b) * (1.0f - wa) + f(c, a + 1, b) * wa) * (1.0f - wb) +
         (f(c, a, b + 1) * (1.0f - wa) + f(c, a + 1, b + 1) * wa) * wb;
}

struct Seg {
  float x0, x1, y0, y1, dx, dy, qvz;
  int ix, iy;
};

// current of one straight segment inside one cell (particles.c:886-922)
template <class D>
__device__ __forceinline__ void deposit_segment(const D &dep, const Seg &v, float qnx, float qny) {
  const float s0x0 = 1.0f - v.x0, s0x1 = v.x0;
  const float s1x0 = 1.0f - v.x1, s1x1 = v.x1;
  const float s0y0 = 1.0f - v.y0, s0y1 = v.y0;
  const float s1y0 = 1.0f - v.y1, s1y1 = v.y1;
  const float jx = qnx * v.dx;
  const float jy = qny * v.dy;
  const float ay0 = 0.5f * (s0y0 + s1y0), ay1 = 0.5f * (s0y1 + s1y1);
  const float ax0 = 0.5f * (s0x0 + s1x0), ax1 = 0.5f * (s0x1 + s1x1);
  dep.add(0, v.ix, v.iy, jx * ay0);
  dep.add(0, v.ix, v.iy + 1, jx * ay1);
  dep.add(1, v.ix, v.iy, jy * ax0);
  dep.add(1, v.ix + 1, v.iy, jy * ax1);
  const float q = v.qvz;
  dep.add(2, v.ix, v.iy, q * (s0x0 * s0y0 + s1x0 * s1y0 + (s0x0 * s1y0 - s1x0 * s0y0) / 2.0f));
  dep.add(2, v.ix + 1, v.iy, q * (s0x1 * s0y0 + s1x1 * s1y0 + (s0x1 * s1y0 - s1x1 * s0y0) / 2.0f));
  dep.add(2, v.ix, v.iy + 1, q * (s0x0 * s0y1 + s1x0 * s1y1 + (s0x0 * s1y1 - s1x0 * s0y1) / 2.0f));
  dep.add(2, v.ix + 1, v.iy + 1, q * (s0x1 * s0y1 + s1x1 * s1y1 + (s0x1 * s1y1 - s1x1 * s0y1) / 2.0f));
}

// splits segment `a` at the y cell edge: `a` keeps the part before the edge,
// the returned segment holds the rest (particles.c:842-871)
__device__ __forceinline__ Seg split_y(Seg &a, int dj) {
  const int yb = (dj == 1);
  const float f = (a.y1 - yb) / a.dy;
  const float xc = a.x0 + a.dx * (1.0f - f);
  Seg n;
  n.y0 = 1 - yb;
  n.y1 = a.y1 - dj;
  n.dy = a.dy * f;
  n.iy = a.iy + dj;
  n.x0 = xc;
  n.x1 = a.x1;
  n.dx = a.dx * f;
  n.ix = a.ix;
  n.qvz = a.qvz * f;
  a.y1 = yb;
  a.dy *= (1.0f - f);
  a.dx *= (1.0f - f);
  a.x1 = xc;
  a.qvz *= (1.0f - f);
  return n;
}

// zigzag deposit of one particle motion (particles.c:773-924), the virtual
// particle cases unrolled so that no per-thread array is indexed
template <class D>
__device__ __forceinline__ void deposit_zigzag(const D &dep, int ix, int iy, int di, int dj, float x0,
                                               float y0, float dx, float dy, float qnx, float qny,
                                               float qvz) {
  Seg a;
  a.x0 = x0;
  a.y0 = y0;
  a.dx = dx;
  a.dy = dy;
  a.x1 = x0 + dx;
  a.y1 = y0 + dy;
  a.qvz = qvz * 0.5f;  // qvz/2.0 in the reference: exact halving either way
  a.ix = ix;
  a.iy = iy;
  if (di == 0 && dj == 0) {
    deposit_segment(dep, a, qnx, qny);
    return;
  }
  if (di != 0) {
    const int xb = (di == 1);
    const float f = (x0 + dx - xb) / dx;
    const float yc = y0 + dy * (1.0f - f);
    Seg b;
    b.x0 = 1 - xb;
    b.x1 = (x0 + dx) - di;
    b.dx = dx * f;
    b.ix = ix + di;
    b.y0 = yc;
    b.y1 = a.y1;
    b.dy = dy * f;
    b.iy = iy;
    b.qvz = a.qvz * f;
    a.x1 = xb;
    a.dx *= (1.0f - f);
    a.dy *= (1.0f - f);
    a.y1 = yc;
    a.qvz *= (1.0f - f);
    if (dj != 0) {
      if (a.y1 < 0.0f || a.y1 >= 1.0f) {
        // the first piece crosses the y edge; the x tail lies past it
        Seg c = split_y(a, dj);
        b.y0 -= dj;
        b.y1 -= dj;
        b.iy += dj;
        deposit_segment(dep, c, qnx, qny);
      } else {
        Seg c = split_y(b, dj);
        deposit_segment(dep, c, qnx, qny);
      }
    }
    deposit_segment(dep, b, qnx, qny);
  } else {
    Seg c = split_y(a, dj);
    deposit_segment(dep, c, qnx, qny);
  }
  deposit_segment(dep, a, qnx, qny);
}

// gather + Boris + move + deposit for one particle at cell (i, j) of the
// accessor frame; returns the kinetic-energy term utsq/(gamma+1).  `bad` is
// set when the motion breaks the one-cell-per-step assumption of the
// deposit (|dx| >= 1 cell, or not a number).  A trimmed position of exactly
// 1.0f (x1 = -tiny, then +1 rounds up) is legal, as in the reference.
template <class F, class D>
__device__ __forceinline__ float advance_particle(const F &fld, const D &dep, int i, int j, float &x,
                                                  float &y, float &ux, float &uy, float &uz, int &di,
                                                  int &dj, bool &bad, const PushConst &C) {
  // staggered bilinear gather (particles.c:1029-1071)
  const int ih = i + ((x < 0.5f) ? -1 : 0);
  const int jh = j + ((y < 0.5f) ? -1 : 0);
  const float w1h = x + ((x < 0.5f) ? 0.5f : -0.5f);
  const float w2h = y + ((y < 0.5f) ? 0.5f : -0.5f);
  float ex = lerp2(fld, 0, ih, j, w1h, y);
  float ey = lerp2(fld, 1, i, jh, x, w2h);
  float ez = lerp2(fld, 2, i, j, x, y);
  float bx = lerp2(fld, 3, i, jh, x, w2h);
  float by = lerp2(fld, 4, ih, j, w1h, y);
  float bz = lerp2(fld, 5, ih, jh, w1h, w2h);

  // relativistic Boris push (particles.c:1145-1187)
  const float tem = C.tem;
  ex *= tem;
  ey *= tem;
  ez *= tem;
  float tx = ux + ex, ty = uy + ey, tz = uz + ez;
  const float u2 = tx * tx + ty * ty + tz * tz;
  const float g = sqrtf(1.0f + u2);
  const float kin = u2 / (g + 1);
  const float tg = tem / g;
  bx *= tg;
  by *= tg;
  bz *= tg;
  const float s2 = 2.0f / (1.0f + bx * bx + by * by + bz * bz);
  float vx = tx + ty * bz - tz * by;
  float vy = ty + tz * bx - tx * bz;
  float vz = tz + tx * by - ty * bx;
  bx *= s2;
  by *= s2;
  bz *= s2;
  tx += vy * bz - vz * by;
  ty += vz * bx - vx * bz;
  tz += vx * by - vy * bx;
  ux = tx + ex;
  uy = ty + ey;
  uz = tz + ez;

  // move and cell crossing (particles.c:1194-1207, ltrim :1081-1084)
  const float rg = 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
  const float mx = C.dt_dx * rg * ux;
  const float my = C.dt_dy * rg * uy;
  bad = !(fabsf(mx) < 1.0f && fabsf(my) < 1.0f);
  float x1 = x + mx, y1 = y + my;
  di = (x1 >= 1.0f) - (x1 < 0.0f);
  dj = (y1 >= 1.0f) - (y1 < 0.0f);
  x1 -= di;
  y1 -= dj;
  const float qvz = C.q * uz * rg;
  deposit_zigzag(dep, i, j, di, dj, x, y, mx, my, C.qnx, C.qny, qvz);
  x = x1;
  y = y1;
  return kin;
}

// new cell after the move, window shift and boundary; false when the
// particle left through an absorbing x boundary (particles.c:1234-1259)
__device__ __forceinline__ bool apply_boundary(int &ix, int &iy, int di, int dj, const PushConst &C) {
  ix += di - C.shift;
  iy += dj;
  iy += ((iy < 0) ? C.ny : 0) - ((iy >= C.ny) ? C.ny : 0);
  if (C.mw) return ix >= 0 && ix < C.nx;
  ix += ((ix < 0) ? C.nx : 0) - ((ix >= C.nx) ? C.nx : 0);
  return true;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

__device__ __forceinline__ void store_particle(const Particles &p, long long k, int ix, int iy, float x,
                                               float y, float ux, float uy, float uz) {
  p.ix[k] = ix;
  p.iy[k] = iy;
  p.x[k] = x;
  p.y[k] = y;
  p.ux[k] = ux;
  p.uy[k] = uy;
  p.uz[k] = uz;
}

__device__ __forceinline__ void spill_particle(const Spill &S, int *errbits, int ix, int iy, float x, float y,
                                               float ux, float uy, float uz) {
  const int q = atomicAdd(S.cnt, 1);
  *errbits |= ERR_SPILLED;
  if (q < S.cap) store_particle(S.p, q, ix, iy, x, y, ux, uy, uz);
  else *errbits |= ERR_OVERFLOW;
}

// ---------------------------------------------------------------------------
// K1: push + deposit, one CTA per tile
// ---------------------------------------------------------------------------
template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_push_tiles(const __grid_constant__ CUtensorMap tm_eb,
                                                   const __grid_constant__ CUtensorMap tm_j, Particles pin,
                                                   Particles pout, TileSet T, Outbox O, Spill S,
                                                   double *ekin_tile, int *err, PushConst C) {
  constexpr int BW = (TX + 3 + 3) & ~3;  // halo box width, multiple of 4 floats
  constexpr int BH = TY + 3;
  constexpr int PL = BW * BH;
  __shared__ __align__(128) float sEB[6 * PL];
  __shared__ __align__(128) float sJ[3 * PL];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int swarp[NT / 32];
  __shared__ double sred[NT / 32];

  const int t = blockIdx.x;
  const int tx = t % C.ntx, ty = t / C.ntx;
  const int cx0 = tx * TX, cy0 = ty * TY;  // first cell of the tile = buffer coords of its halo
  int errbits = 0;

  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, 6 * PL * 4);
    tma_load_3d(sEB, &tm_eb, cx0, cy0, 0, &bar);
  }
  for (int k = threadIdx.x; k < 3 * PL; k += NT) sJ[k] = 0.f;
  const bool loaded = mbar_wait_bounded(&bar, 0);
  if (!loaded) errbits |= ERR_TIMEOUT;
  __syncthreads();

  const TileFields<BW, PL> fld{sEB};
  const TileCurrent<BW, PL> dep{sJ};
  const long long base = T.off[t];
  const int n = T.np[t];
  const long long obase = (long long)t * O.cap;
  int run_stay = 0, run_leave = 0;
  float ks = 0.f, kc = 0.f;

  for (int k0 = 0; k0 < n; k0 += NT) {
    const int k = k0 + threadIdx.x;
    int code = 0;  // 1 stays in the tile, 2 leaves it
    int ix = 0, iy = 0, dest = 0;
    float x = 0.f, y = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
    if (k < n) {
      const long long g = base + k;
      ix = pin.ix[g];
      iy = pin.iy[g];
      x = pin.x[g];
      y = pin.y[g];
      ux = pin.ux[g];
      uy = pin.uy[g];
      uz = pin.uz[g];
      int li = ix - cx0, lj = iy - cy0;
      if ((unsigned)li >= (unsigned)TX || (unsigned)lj >= (unsigned)TY) {
        errbits |= ERR_ESCAPE;  // not in this tile: keep the accesses inside the halo
        li = min(max(li, 0), TX - 1);
        lj = min(max(lj, 0), TY - 1);
        ix = cx0 + li;
        iy = cy0 + lj;
      }
      int di, dj;
      bool bad;
      const float kin = advance_particle(fld, dep, li, lj, x, y, ux, uy, uz, di, dj, bad, C);
      kahan_add(ks, kc, kin);
      if (bad) errbits |= ERR_ESCAPE;
      if (apply_boundary(ix, iy, di, dj, C)) {
        dest = ix / TX + (iy / TY) * C.ntx;
        code = (dest == t) ? 1 : 2;
      }
    }
    int tot;
    const int pre = block_exclusive_scan<NT>((code == 1) | ((code == 2) << 16), tot, swarp);
    if (code == 1) {
      store_particle(pout, base + run_stay + (pre & 0xffff), ix, iy, x, y, ux, uy, uz);
    } else if (code == 2) {
      const int s = run_leave + (pre >> 16);
      if (s < O.cap) {
        store_particle(O.p, obase + s, ix, iy, x, y, ux, uy, uz);
        O.dst[obase + s] = dest;
      } else {
        spill_particle(S, &errbits, ix, iy, x, y, ux, uy, uz);
      }
    }
    run_stay += tot & 0xffff;
    run_leave += tot >> 16;
  }

  if (threadIdx.x == 0) {
    T.nstay[t] = run_stay;
    O.cnt[t] = min(run_leave, O.cap);
  }
  const double e = block_sum_double<NT>((double)ks - (double)kc, sred);
  if (threadIdx.x == 0) ekin_tile[t] = e;

  // all shared-memory atomics done: hand the J tile to the TMA unit
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    if (loaded) {
      tma_reduce_add_3d(&tm_j, sJ, cx0, cy0, 0);
      bulk_commit();
      bulk_wait_read0();
    } else if (!mbar_wait_bounded(&bar, 0)) {
      errbits |= ERR_TIMEOUT;  // second bounded wait for the load still in flight
    }
  }
  if (errbits) atomicOr(err, errbits);
}

// ---------------------------------------------------------------------------
// spill push: same physics from global memory (rarely non-empty)
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT) k_push_spill(const float *EB, float *J, Grid G, Particles sin,
                                                   const int *sin_cnt, int sin_cap, Spill S, double *ekin,
                                                   int *err, PushConst C) {
  __shared__ double sred[NT / 32];
  const int n = min(*sin_cnt, sin_cap);
  const GlobalFields fld{EB, G.pitch, G.plane};
  const GlobalCurrent dep{J, G.pitch, G.plane};
  int errbits = 0;
  float ks = 0.f, kc = 0.f;
  for (int k = blockIdx.x * NT + threadIdx.x; k < n; k += gridDim.x * NT) {
    int ix = sin.ix[k], iy = sin.iy[k];
    float x = sin.x[k], y = sin.y[k], ux = sin.ux[k], uy = sin.uy[k], uz = sin.uz[k];
    if (ix < 0 || ix >= C.nx || iy < 0 || iy >= C.ny) {
      errbits |= ERR_ESCAPE;
      ix = min(max(ix, 0), C.nx - 1);
      iy = min(max(iy, 0), C.ny - 1);
    }
    int di, dj;
    bool bad;
    const float kin = advance_particle(fld, dep, ix, iy, x, y, ux, uy, uz, di, dj, bad, C);
    if (bad) errbits |= ERR_ESCAPE;
    kahan_add(ks, kc, kin);
    if (apply_boundary(ix, iy, di, dj, C)) spill_particle(S, &errbits, ix, iy, x, y, ux, uy, uz);
  }
  const double e = block_sum_double<NT>((double)ks - (double)kc, sred);
  if (threadIdx.x == 0 && e != 0.0) atomicAdd(ekin, e);
  if (errbits) atomicOr(err, errbits);
}

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
  const int stay = T.nstay[t];
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
          store_particle(pout, start + s, O.p.ix[q], O.p.iy[q], O.p.x[q], O.p.y[q], O.p.ux[q], O.p.uy[q],
                         O.p.uz[q]);
        else
          spill_particle(S, &errbits, O.p.ix[q], O.p.iy[q], O.p.x[q], O.p.y[q], O.p.ux[q], O.p.uy[q],
                         O.p.uz[q]);
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

// AoS staging records -> SoA list, counting the particles of each tile
__global__ void k_stage_to_list(const float4 *aos7, int n, Particles list, int *cnt, LayoutConst L,
                                int *err) {
  // records are 7 words; read them as words
  const int *w = reinterpret_cast<const int *>(aos7);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int *r = w + 7LL * k;
    int ix = r[0], iy = r[1];
    if (ix < 0 || ix >= L.nx || iy < 0 || iy >= L.ny) {
      atomicOr(err, ERR_ESCAPE);
      ix = min(max(ix, 0), L.nx - 1);
      iy = min(max(iy, 0), L.ny - 1);
    }
    list.ix[k] = ix;
    list.iy[k] = iy;
    list.x[k] = __int_as_float(r[2]);
    list.y[k] = __int_as_float(r[3]);
    list.ux[k] = __int_as_float(r[4]);
    list.uy[k] = __int_as_float(r[5]);
    list.uz[k] = __int_as_float(r[6]);
    atomicAdd(&cnt[tile_of(ix, iy, L)], 1);
  }
}

// counts the particles of a list per tile (list length read on the device)
__global__ void k_count_list(Particles list, const int *n_ptr, int n_cap, int *cnt, LayoutConst L) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    atomicAdd(&cnt[tile_of(list.ix[k], list.iy[k], L)], 1);
}

// tile particles keep their tile and their order: copy to the new offsets
__global__ void k_copy_tiles(Particles src, const int *off_old, const int *np_old, Particles dst,
                             const int *off_new, unsigned *key, int *fill) {
  const int t = blockIdx.x;
  const int n = np_old[t];
  const long long a = off_old[t], b = off_new[t];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    store_particle(dst, b + k, src.ix[a + k], src.iy[a + k], src.x[a + k], src.y[a + k], src.ux[a + k],
                   src.uy[a + k], src.uz[a + k]);
    if (key) key[b + k] = (unsigned)k;
  }
  if (threadIdx.x == 0) fill[t] = n;
}

// list particles are appended to their tile; `key0 + k` remembers the order
__global__ void k_scatter_list(Particles list, const int *n_ptr, int n_cap, Particles dst, const int *off,
                               const int *cap, int *fill, unsigned *key, unsigned key0, LayoutConst L,
                               int *err) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int t = tile_of(list.ix[k], list.iy[k], L);
    const int s = atomicAdd(&fill[t], 1);
    if (s < cap[t]) {
      const long long q = (long long)off[t] + s;
      store_particle(dst, q, list.ix[k], list.iy[k], list.x[k], list.y[k], list.ux[k], list.uy[k],
                     list.uz[k]);
      if (key) key[q] = key0 + (unsigned)k;
    } else {
      atomicOr(err, ERR_OVERFLOW);  // capacities are sized from exact counts: cannot happen
    }
  }
}

// Orders every tile deterministically: sort by key (origin order), then
// interleave with stride P so that neighbouring threads of the push kernel
// work on particles of different cells (fewer shared-memory atomic
// collisions).  One CTA per tile; tiles larger than the shared-memory sort
// capacity are copied in key-unsorted order.
__global__ void k_tile_order(Particles src, const unsigned *key, const int *off, const int *np,
                             Particles dst, int smax, int stride_p) {
  extern __shared__ unsigned long long sk[];  // (key << 32) | local index
  const int t = blockIdx.x;
  const int n = np[t];
  const long long b = off[t];
  if (n <= smax) {
    int m = 1;
    while (m < n) m <<= 1;
    for (int k = threadIdx.x; k < m; k += blockDim.x)
      sk[k] = (k < n) ? (((unsigned long long)key[b + k] << 32) | (unsigned)k) : ~0ull;
    __syncthreads();
    for (int size = 2; size <= m; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
          const int o = k ^ stride;
          if (o > k) {
            const bool up = ((k & size) == 0);
            const unsigned long long a = sk[k], c = sk[o];
            if ((a > c) == up) {
              sk[k] = c;
              sk[o] = a;
            }
          }
        }
        __syncthreads();
      }
  }
  const int P = stride_p;
  const int q = n / P, r = n % P;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const int from = (n <= smax) ? (int)(sk[p] & 0xffffffffu) : p;
    const int res = p % P;
    const int to = res * q + min(res, r) + p / P;
    const long long s = b + from, d = b + to;
    store_particle(dst, d, src.ix[s], src.iy[s], src.x[s], src.y[s], src.ux[s], src.uy[s], src.uz[s]);
  }
}

// appends a list to the tiles in place (moving-window injection); overflow
// goes to the spill list that the next push processes
__global__ void k_append_list(Particles list, int n, Particles buf, TileSet T, Spill S, LayoutConst L,
                              int *err) {
  int errbits = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int ix = list.ix[k], iy = list.iy[k];
    if (ix < 0 || ix >= L.nx || iy < 0 || iy >= L.ny) {
      errbits |= ERR_ESCAPE;
      continue;
    }
    const int t = tile_of(ix, iy, L);
    const int s = atomicAdd(&T.np[t], 1);
    if (s < T.cap[t])
      store_particle(buf, (long long)T.off[t] + s, ix, iy, list.x[k], list.y[k], list.ux[k], list.uy[k],
                     list.uz[k]);
    else
      spill_particle(S, &errbits, ix, iy, list.x[k], list.y[k], list.ux[k], list.uy[k], list.uz[k]);
  }
  if (errbits) atomicOr(err, errbits);
}

__global__ void k_clamp_counts(int *np, const int *cap, int ntiles) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
    np[t] = min(np[t], cap[t]);
}

// tiles + spill -> AoS records in tile order (download)
__global__ void k_gather_aos(Particles buf, const int *off, const int *np, const long long *dst_off,
                             int *aos, int ntiles) {
  const int t = blockIdx.x;
  if (t >= ntiles) return;
  const int n = np[t];
  const long long a = off[t], d = dst_off[t];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    int *r = aos + 7LL * (d + k);
    r[0] = buf.ix[a + k];
    r[1] = buf.iy[a + k];
    r[2] = __float_as_int(buf.x[a + k]);
    r[3] = __float_as_int(buf.y[a + k]);
    r[4] = __float_as_int(buf.ux[a + k]);
    r[5] = __float_as_int(buf.uy[a + k]);
    r[6] = __float_as_int(buf.uz[a + k]);
  }
}

__global__ void k_list_to_aos(Particles list, const int *n_ptr, int n_cap, int *aos, long long d0) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int *r = aos + 7LL * (d0 + k);
    r[0] = list.ix[k];
    r[1] = list.iy[k];
    r[2] = __float_as_int(list.x[k]);
    r[3] = __float_as_int(list.y[k]);
    r[4] = __float_as_int(list.ux[k]);
    r[5] = __float_as_int(list.uy[k]);
    r[6] = __float_as_int(list.uz[k]);
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
    const int c = buf.ix[a + k] + nrow * buf.iy[a + k];
    const float w1 = buf.x[a + k], w2 = buf.y[a + k];
    atomicAdd(&rho[c], (1.0f - w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + 1], (w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + nrow], (1.0f - w1) * (w2) * q);
    atomicAdd(&rho[c + 1 + nrow], (w1) * (w2) * q);
  }
}

__global__ void k_charge_list(Particles list, const int *n_ptr, int n_cap, float *rho, int nrow, float q) {
  const int n = min(*n_ptr, n_cap);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int c = list.ix[k] + nrow * list.iy[k];
    const float w1 = list.x[k], w2 = list.y[k];
    atomicAdd(&rho[c], (1.0f - w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + 1], (w1) * (1.0f - w2) * q);
    atomicAdd(&rho[c + nrow], (1.0f - w1) * (w2) * q);
    atomicAdd(&rho[c + 1 + nrow], (w1) * (w2) * q);
  }
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
                             float dx, float dy) {
  __shared__ double sred[8];
  double s = 0;
  for (int t = threadIdx.x; t < ntiles; t += 256) s += tiles[t];
  s = block_sum_double<256>(s, sred);
  if (threadIdx.x == 0) {
    s += *extra;
    // spec->energy = q * m_q * energy * dx * dy  (particles.c:1231)
    *out = scale_q_mq * s * dx * dy;
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <int TX, int TY>
static cudaError_t launch_push_t(const PushLaunch &a, cudaStream_t st) {
  constexpr int NT = (TX * TY >= 256) ? 256 : 128;
  k_push_tiles<TX, TY, NT><<<a.ntiles, NT, 0, st>>>(*a.tm_eb, *a.tm_j, a.pin, a.pout, a.T, a.O, a.S,
                                                     a.ekin_tile, a.err, a.C);
  return cudaGetLastError();
}

cudaError_t launch_push_tiles(const PushLaunch &a, cudaStream_t st) {
  const int TX = a.TX, TY = a.TY;
#define ZC_TILE(X, Y) \
  if (TX == X && TY == Y) return launch_push_t<X, Y>(a, st);
  ZC_TILE(16, 16)
  ZC_TILE(8, 8)
  ZC_TILE(16, 8)
  ZC_TILE(32, 16)
  ZC_TILE(32, 32)
  ZC_TILE(8, 16)
  ZC_TILE(16, 32)
#undef ZC_TILE
  return cudaErrorInvalidValue;
}

bool tile_supported(int TX, int TY) {
  return (TX == 16 && TY == 16) || (TX == 8 && TY == 8) || (TX == 16 && TY == 8) || (TX == 32 && TY == 16) ||
         (TX == 32 && TY == 32) || (TX == 8 && TY == 16) || (TX == 16 && TY == 32);
}

cudaError_t launch_push_spill(const float *EB, float *J, const Grid &G, const Particles &sin, const int *sin_cnt,
                              int sin_cap, const Spill &S, double *ekin, int *err, const PushConst &C,
                              int nblocks, cudaStream_t st) {
  k_push_spill<256><<<nblocks, 256, 0, st>>>(EB, J, G, sin, sin_cnt, sin_cap, S, ekin, err, C);
  return cudaGetLastError();
}

cudaError_t launch_migrate(const Particles &pout, const TileSet &T, const Outbox &O, const Spill &S, int *err,
                           int ntx, int nty, int mw, cudaStream_t st) {
  k_migrate<256><<<ntx * nty, 256, 0, st>>>(pout, T, O, S, err, ntx, nty, mw);
  return cudaGetLastError();
}

cudaError_t launch_stage_to_list(const void *aos, int n, const Particles &list, int *cnt, const LayoutConst &L,
                                 int *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = (int)std::min<long long>((n + 255) / 256, 4096);
  k_stage_to_list<<<nb, 256, 0, st>>>(reinterpret_cast<const float4 *>(aos), n, list, cnt, L, err);
  return cudaGetLastError();
}

cudaError_t launch_count_list(const Particles &list, const int *n_ptr, int n_cap, int *cnt, const LayoutConst &L,
                              cudaStream_t st) {
  k_count_list<<<256, 256, 0, st>>>(list, n_ptr, n_cap, cnt, L);
  return cudaGetLastError();
}

cudaError_t launch_copy_tiles(const Particles &src, const int *off_old, const int *np_old, const Particles &dst,
                              const int *off_new, unsigned *key, int *fill, int ntiles, cudaStream_t st) {
  k_copy_tiles<<<ntiles, 256, 0, st>>>(src, off_old, np_old, dst, off_new, key, fill);
  return cudaGetLastError();
}

cudaError_t launch_scatter_list(const Particles &list, const int *n_ptr, int n_cap, const Particles &dst,
                                const int *off, const int *cap, int *fill, unsigned *key, unsigned key0,
                                const LayoutConst &L, int *err, cudaStream_t st) {
  k_scatter_list<<<512, 256, 0, st>>>(list, n_ptr, n_cap, dst, off, cap, fill, key, key0, L, err);
  return cudaGetLastError();
}

cudaError_t launch_tile_order(const Particles &src, const unsigned *key, const int *off, const int *np,
                              const Particles &dst, int ntiles, int smax, int stride_p, cudaStream_t st) {
  const size_t sh = (size_t)smax * sizeof(unsigned long long);
  if (sh > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_tile_order, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    if (e != cudaSuccess) return e;
  }
  k_tile_order<<<ntiles, 1024, sh, st>>>(src, key, off, np, dst, smax, stride_p);
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
                              float dx, float dy, cudaStream_t st) {
  k_sum_energy<<<1, 256, 0, st>>>(tiles, ntiles, extra, out, q_mq, dx, dy);
  return cudaGetLastError();
}

}  // namespace zc
