// zc_push_impl.cuh -- particle push + current deposit kernels.
//
// Included twice, inside namespaces zc::exact and zc::fast, by
// zc_push_exact.cu (compiled with --fmad=false and IEEE division / square
// root: every float32 operation rounds as in the reference C, particles
// advanced from the same fields land on the same bits) and zc_push_fast.cu
// (FMA contraction and the hardware's approximate float32 division and
// square root: same algorithm, results within a few float32 ulps per
// operation of the exact build).
//
//   k_push_tiles  one CTA per particle tile (TX x TY cells).  The tile's E/B
//                 with a 1-lower / 2-upper cell halo arrive in shared memory
//                 by one 3-D TMA box; every particle of the tile is pushed
//                 (staggered bilinear gather, relativistic Boris, move) and
//                 its current deposited with the zigzag scheme.  Tiles are
//                 kept sorted by cell, so the lanes of a warp mostly share a
//                 cell: their gathers are broadcasts, and the current of the
//                 segment every particle starts with (it lies in the
//                 particle's own cell) is summed across the lanes of a cell
//                 with a segmented warp-shuffle reduction before one lane per
//                 cell deposits it.  The fast and exact builds deposit with
//                 float reductions on the global J planes, which L2 performs
//                 natively; the deterministic builds accumulate a shared
//                 integer J tile (exact, order-independent sums) and add it
//                 to the global fixed-point planes.  Cell-crossing motions (a
//                 few per cent) wait in a per-warp shared-memory queue and are
//                 split and deposited a warp's worth at a time, so the split
//                 code runs with (nearly) full warps.  Particles that stay
//                 are compacted in order; particles that leave go to the
//                 tile's outbox, from which the destination tile pulls them
//                 at the start of the next step's push.
//   k_push_spill  the same physics for particles that did not fit a tile,
//                 from global memory (normally empty).
//
// Requires zc_internal.cuh and zc_kernels.h to be included first.

// ---------------------------------------------------------------------------
// field / current accessors: shared-memory tile (1-cell lower halo) or the
// global padded planes
// ---------------------------------------------------------------------------
template <int BW, int PL>
struct TileFields {
  const float *s;
  __device__ __forceinline__ float operator()(int c, int i, int j) const {
    return s[c * PL + (j + 1) * BW + (i + 1)];
  }
};
// The tile current is kept as three planes of 32-bit integers: a
// contribution v counts as the integer rint(v js) = h 2^2L + m 2^L + l (js a
// power of two, |m|, |l| <= 2^(L-1)), each part added to its plane with a
// 32-bit integer atomic (float atomic adds on shared memory run as
// compare-and-swap loops, integer ones are single instructions).  The host
// picks L so that no plane can overflow with the most contributions a tile
// can take, and js = 2^40 (the unit of the deterministic mode) unless the
// largest contribution needs a smaller one.  The parts are rounded with the
// 1.5 2^23 shifter (exact for |t| < 2^22) instead of conversion instructions.
constexpr float kShifter = 12582912.0f;  // 1.5 * 2^23
constexpr int kShifterBits = 0x4B400000;

__device__ __forceinline__ void jsplit(float v, const PushConst &C, int &h, int &m, int &l) {
  const float x = __fmul_rn(v, C.js);                  // exact: js is a power of two
  const float th = __fmaf_rn(x, C.js_inv2l, kShifter);  // rint(x 2^-2L) + shifter
  h = __float_as_int(th) - kShifterBits;
  const float r1 = __fmaf_rn(-__fsub_rn(th, kShifter), C.js_two2l, x);  // exact remainder
  const float tm = __fmaf_rn(r1, C.js_invl, kShifter);
  m = __float_as_int(tm) - kShifterBits;
  const float r2 = __fmaf_rn(-__fsub_rn(tm, kShifter), C.js_twol, r1);  // exact remainder
  l = __float_as_int(__fadd_rn(r2, kShifter)) - kShifterBits;
}

// node offsets of the integer J tile, per component: Jx takes columns
// -1..TX, Jy rows -1..TY, Jz both one more (the halo each can receive)
template <int TX, int TY>
struct JTileLayout {
  static constexpr int WX = TX + 2, HX = TY + 3;
  static constexpr int WY = TX + 3, HY = TY + 2;
  static constexpr int WZ = TX + 3, HZ = TY + 3;
  static constexpr int OX = 0, OY = WX * HX, OZ = OY + WY * HY;
  static constexpr int N = OZ + WZ * HZ;  // nodes per plane
  // component, row and column (halo included) of node k
  __device__ __forceinline__ static void where(int k, int &c, int &r, int &col) {
    if (k < OY) {
      c = 0, r = k / WX, col = k % WX;
    } else if (k < OZ) {
      c = 1, r = (k - OY) / WY, col = (k - OY) % WY;
    } else {
      c = 2, r = (k - OZ) / WZ, col = (k - OZ) % WZ;
    }
  }
  __device__ __forceinline__ static int node(int c, int i, int j) {
    return c == 0 ? OX + (j + 1) * WX + (i + 1) : (c == 1 ? OY + (j + 1) * WY + (i + 1) : OZ + (j + 1) * WZ + (i + 1));
  }
};

// fast and exact builds: every deposit goes straight to the global J
// planes as a float reduction, which L2 performs (no compare-and-swap loop);
// g points at the tile's first cell, (i, j) run over -1 .. TX, -1 .. TY
struct TileCurrentGlobal {
  float *g;
  int pitch;
  size_t plane;
  __device__ __forceinline__ void add(int c, int i, int j, float v) const {
    atomicAdd(g + c * plane + (long long)j * pitch + i, v);
  }
};

// the integer a node of the tile holds: h 2^2L + m 2^L + l
__device__ __forceinline__ long long tile_node_sum(const int *p, int n, int k, int L) {
  return (long long)p[k] * (1LL << (2 * L)) + (long long)p[n + k] * (1LL << L) + p[2 * n + k];
}

template <class LAY>
struct TileCurrentSplit {
  int *p;  // planes h, m, l of LAY::N nodes each
  const PushConst *C;
  __device__ __forceinline__ void add(int c, int i, int j, float v) const {
    int h, m, l;
    jsplit(v, *C, h, m, l);
    addi(c, i, j, h, m, l);
  }
  __device__ __forceinline__ void addi(int c, int i, int j, int h, int m, int l) const {
    const int k = LAY::node(c, i, j);
    atomicAdd(&p[k], h);
    atomicAdd(&p[LAY::N + k], m);
    atomicAdd(&p[2 * LAY::N + k], l);
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

// deterministic mode: every contribution rounded once to the integer
// rint(v js) (as the tile current rounds it) and summed in units of 2^-40
__device__ __forceinline__ long long to_fixed(float v, const PushConst &C) {
  return __float2ll_rn(v * C.js) * C.js_det;
}

struct GlobalCurrentFixed {
  unsigned long long *g;
  int pitch;
  size_t plane;
  const PushConst *C;
  __device__ __forceinline__ void add(int c, int i, int j, float v) const {
    atomicAdd(&g[c * plane + (size_t)(j + 1) * pitch + (i + 1)], (unsigned long long)to_fixed(v, *C));
  }
};

// ---------------------------------------------------------------------------
// per-particle physics (restates em2d/particles.c:773-924, 1029-1226)
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

// the 8 current contributions of one straight segment inside one cell
// (particles.c:886-922): Jx at (ix,iy),(ix,iy+1); Jy at (ix,iy),(ix+1,iy);
// Jz at the four corners (ix,iy),(ix+1,iy),(ix,iy+1),(ix+1,iy+1)
struct SegCurrent {
  float v[8];
};

__device__ __forceinline__ SegCurrent segment_current(const Seg &s, float qnx, float qny) {
#ifdef ZC_FAST_ALGEBRA
  // the same weights, re-associated (fast build only): Jx, Jy from the
  // segment's mid-point; each Jz corner q (a (c + d/2) + b (d - c/2)) with
  // a, b its start / end x weights and c, d its start / end y weights
  SegCurrent r;
  const float jx = qnx * s.dx, jy = qny * s.dy;
  const float ym = 0.5f * (s.y0 + s.y1), xm = 0.5f * (s.x0 + s.x1);
  r.v[1] = jx * ym;
  r.v[0] = jx - r.v[1];
  r.v[3] = jy * xm;
  r.v[2] = jy - r.v[3];
  const float c0 = 1.0f - s.y0, d0 = 1.0f - s.y1;
  const float p0 = c0 + 0.5f * d0, m0 = d0 - 0.5f * c0;
  const float p1 = s.y0 + 0.5f * s.y1, m1 = s.y1 - 0.5f * s.y0;
  const float a0 = 1.0f - s.x0, b0 = 1.0f - s.x1;
  const float q = s.qvz;
  r.v[4] = q * (a0 * p0 + b0 * m0);
  r.v[5] = q * (s.x0 * p0 + s.x1 * m0);
  r.v[6] = q * (a0 * p1 + b0 * m1);
  r.v[7] = q * (s.x0 * p1 + s.x1 * m1);
  return r;
#else
  const float s0x0 = 1.0f - s.x0, s0x1 = s.x0;
  const float s1x0 = 1.0f - s.x1, s1x1 = s.x1;
  const float s0y0 = 1.0f - s.y0, s0y1 = s.y0;
  const float s1y0 = 1.0f - s.y1, s1y1 = s.y1;
  const float jx = qnx * s.dx;
  const float jy = qny * s.dy;
  const float ay0 = 0.5f * (s0y0 + s1y0), ay1 = 0.5f * (s0y1 + s1y1);
  const float ax0 = 0.5f * (s0x0 + s1x0), ax1 = 0.5f * (s0x1 + s1x1);
  const float q = s.qvz;
  SegCurrent r;
  r.v[0] = jx * ay0;
  r.v[1] = jx * ay1;
  r.v[2] = jy * ax0;
  r.v[3] = jy * ax1;
  r.v[4] = q * (s0x0 * s0y0 + s1x0 * s1y0 + (s0x0 * s1y0 - s1x0 * s0y0) / 2.0f);
  r.v[5] = q * (s0x1 * s0y0 + s1x1 * s1y0 + (s0x1 * s1y0 - s1x1 * s0y0) / 2.0f);
  r.v[6] = q * (s0x0 * s0y1 + s1x0 * s1y1 + (s0x0 * s1y1 - s1x0 * s0y1) / 2.0f);
  r.v[7] = q * (s0x1 * s0y1 + s1x1 * s1y1 + (s0x1 * s1y1 - s1x1 * s0y1) / 2.0f);
  return r;
#endif
}

template <class D>
__device__ __forceinline__ void add_current(const D &dep, int ix, int iy, const SegCurrent &c) {
  dep.add(0, ix, iy, c.v[0]);
  dep.add(0, ix, iy + 1, c.v[1]);
  dep.add(1, ix, iy, c.v[2]);
  dep.add(1, ix + 1, iy, c.v[3]);
  dep.add(2, ix, iy, c.v[4]);
  dep.add(2, ix + 1, iy, c.v[5]);
  dep.add(2, ix, iy + 1, c.v[6]);
  dep.add(2, ix + 1, iy + 1, c.v[7]);
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

// Zigzag trajectory split (particles.c:773-879): returns the first segment,
// which always starts in the particle's own cell; the (at most two) further
// segments of a cell-crossing motion are deposited right away.
template <class D>
__device__ __forceinline__ Seg zigzag_first(const D &dep, int ix, int iy, int di, int dj, float x0, float y0,
                                            float dx, float dy, float qnx, float qny, float qvz) {
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
        const Seg c = split_y(a, dj);
        b.y0 -= dj;
        b.y1 -= dj;
        b.iy += dj;
        add_current(dep, c.ix, c.iy, segment_current(c, qnx, qny));
      } else {
        const Seg c = split_y(b, dj);
        add_current(dep, c.ix, c.iy, segment_current(c, qnx, qny));
      }
    }
    add_current(dep, b.ix, b.iy, segment_current(b, qnx, qny));
  } else if (dj != 0) {
    const Seg c = split_y(a, dj);
    add_current(dep, c.ix, c.iy, segment_current(c, qnx, qny));
  }
  return a;
}

// gather + Boris + move for one particle at cell (i, j) of the accessor
// frame (particles.c:1029-1207); leaves the displacement in (mx, my) and the
// cell shift in (di, dj), returns the kinetic-energy term utsq/(gamma+1).
// `bad` flags a motion of one cell or more (or NaN), which the deposit does
// not support.  A trimmed position of exactly 1.0f (x1 = -tiny, +1 rounds up)
// is legal, as in the reference.
template <class F>
__device__ __forceinline__ float push_particle(const F &fld, int i, int j, float &x, float &y, float &ux,
                                               float &uy, float &uz, float &mx, float &my, float &x1, float &y1,
                                               int &di, int &dj, float &qvz, bool &bad, const PushConst &C) {
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

  const float rg = 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
  mx = C.dt_dx * rg * ux;
  my = C.dt_dy * rg * uy;
  bad = !(fabsf(mx) < 1.0f && fabsf(my) < 1.0f);
  x1 = x + mx;
  y1 = y + my;
  di = (x1 >= 1.0f) - (x1 < 0.0f);
  dj = (y1 >= 1.0f) - (y1 < 0.0f);
  x1 -= di;
  y1 -= dj;
  qvz = C.q * uz * rg;
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

// ---------------------------------------------------------------------------
// K1: push + deposit, one CTA per tile.  The input of tile t is its own
// slots plus the particles that the previous step posted for it in the
// outboxes of its (up to 8) neighbouring tiles (`Oin`); leavers of this step
// go to this tile's slot of `O`.
//
// Own particles keep their slots: each is written back to the slot it was
// read from (a particle that leaves writes a hole there), so the cell order
// the sort gave the tile survives until the next sort except for the few
// particles that change cell.  The particles bound for the tile are listed
// from the neighbours' outboxes (one warp per neighbour), pushed in full
// warps after the own ones and appended after slot np.  The main loop has
// no block-wide barrier.
//
// Warp w takes the chunks w, w + NW, ... of kChunk slots, 32 slots at a
// time.  In the float builds lane l meets the chunk's particles l kLaneRun
// ... l kLaneRun + kLaneRun - 1 of the sorted order one after another, and
// sums their single-segment currents in registers while they stay in one
// cell; a lane adds its sums to J when its cell changes.  The deterministic
// builds read every chunk in cell order across the lanes and pre-reduce
// with segmented warp sums of fixed-point parts.
// ---------------------------------------------------------------------------
// resident CTAs per SM the float builds are compiled for: 7 (up to 72
// registers a thread) measured faster than 8 (64, with spills) and 6
#ifndef ZC_PUSH_MIN_CTAS
#define ZC_PUSH_MIN_CTAS 7
#endif
template <int TX, int TY, int NT, bool DET>
__global__ void __launch_bounds__(NT, DET ? 1024 / NT : ZC_PUSH_MIN_CTAS) k_push_tiles(const __grid_constant__ CUtensorMap tm_eb,
                                                   Particles pin,
                                                   Particles pout, TileSet T, Outbox Oin, Outbox O, Spill S,
                                                   double *ekin_tile, int *err, PushConst C, FixedJ fj) {
  constexpr int BW = (TX + 3 + 3) & ~3;  // halo box width, multiple of 4 floats
  constexpr int BH = TY + 3;
  constexpr int PL = BW * BH;
  constexpr int NW = NT / 32;
  using LAY = JTileLayout<TX, TY>;
  __shared__ __align__(128) float sEB[6 * PL];  // E/B tile with its halo
  // deterministic builds: J tile, integer parts h, m, l (jsplit)
  __shared__ __align__(16) int sJi[DET ? 3 * LAY::N : 1];
  __shared__ unsigned long long s_ekin[2];                // fixed-point kinetic energy (DET)
  __shared__ __align__(8) uint64_t bar;
  __shared__ double sred[NW];
  // per-warp queue of cell-crossing motions, deposited 32 at a time so that
  // the split code runs with (nearly) full warps: flushed from QFLUSH
  // waiting motions on, so at most QFLUSH - 1 + 32 are held
  constexpr int QFLUSH = DET ? 24 : 32;
  constexpr int QCAP = QFLUSH - 1 + 32;
  __shared__ float qf[NW][5][QCAP];  // x0, y0, dx, dy, qvz
  __shared__ int qi[NW][QCAP];       // local cell and shifts, packed
  // prefetched particles, 32 slots per warp: each lane reads its slot into
  // registers before it copies the next slot's particle into it
  __shared__ __align__(16) float4 pf_u[NW][32];
  __shared__ __align__(16) float2 pf_xy[NW][32];
  __shared__ int nb[8], s_nnb;        // distinct neighbour tiles
  // incoming particles bound for this tile, listed as (outbox slot << 4 |
  // neighbour) so that they are pushed in full warps
  constexpr int INCAP = 64;
  __shared__ int s_in[INCAP];
  __shared__ int s_nin;
  __shared__ int s_app, s_leave;      // appended arrivals, leavers (warp-aggregated atomics)

  const int t = blockIdx.x;
  const int tx = t % C.ntx, ty = t / C.ntx;
  const int cx0 = tx * TX, cy0 = ty * TY;  // first cell of the tile = buffer coords of its halo
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1;
  int errbits = 0;
  int qcount = 0;  // warp-uniform

  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    int c = 0;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy) continue;
        int x = tx + dx, y = ty + dy;
        y += (y < 0) ? C.nty : 0;
        y -= (y >= C.nty) ? C.nty : 0;
        if (x < 0 || x >= C.ntx) {
          if (C.mw) continue;
          x = (x + C.ntx) % C.ntx;
        }
        const int id = x + y * C.ntx;
        bool dup = (id == t);
        for (int m = 0; m < c; ++m) dup |= (nb[m] == id);
        if (!dup) nb[c++] = id;
      }
    s_nnb = c;
    s_nin = 0;
    s_app = 0;
    s_leave = 0;
    s_ekin[0] = 0;
    s_ekin[1] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, 6 * PL * 4);
    tma_load_3d(sEB, &tm_eb, cx0, cy0, 0, &bar);
  }
  if constexpr (DET)
    for (int k = threadIdx.x; k < 3 * LAY::N; k += NT) sJi[k] = 0;
  const bool loaded = mbar_wait_bounded(&bar, 0);
  if (!loaded) errbits |= ERR_TIMEOUT;
  __syncthreads();

  const TileFields<BW, PL> fld{sEB};
  const PushConst Cl = C;
  const auto dep = [&] {
    if constexpr (DET)
      return TileCurrentSplit<LAY>{sJi, &Cl};
    else
      return TileCurrentGlobal{fj.f + (size_t)(cy0 + 1) * fj.pitch + (cx0 + 1), fj.pitch, fj.plane};
  }();
  const long long base = T.off[t];
  const int cap = T.cap[t];
  const int n_own = T.np[t];
  const long long obase = (long long)t * O.cap;
  const int nnb = s_nnb;
  float ks = 0.f, kc = 0.f;
  long long khi = 0, klo = 0;  // DET: fixed-point kinetic energy of this thread's particles
  // float builds: this lane's running single-segment current and its local
  // cell (-1: none)
  SegCurrent acc;
#pragma unroll
  for (int q = 0; q < 8; ++q) acc.v[q] = 0.f;
  int acc_key = -1;

  // deposits queued motion e of this warp (all segments, direct atomics)
  auto deposit_queued = [&](int e) {
    const int w = qi[warp][e];
    const int qli = w & 0xff, qlj = (w >> 8) & 0xff, qdi = ((w >> 16) & 3) - 1, qdj = ((w >> 18) & 3) - 1;
    const Seg a = zigzag_first(dep, qli, qlj, qdi, qdj, qf[warp][0][e], qf[warp][1][e], qf[warp][2][e],
                               qf[warp][3][e], Cl.qnx, Cl.qny, qf[warp][4][e]);
    add_current(dep, a.ix, a.iy, segment_current(a, Cl.qnx, Cl.qny));
  };

  // one particle per lane: push, deposit, boundary, output; the 32 lanes of
  // a warp call it together (warp-level collectives only).  `oslot` is the
  // lane's own slot (>= 0: the output goes back there, a particle or a
  // hole) or negative (no own slot); `incoming` marks arriving particles,
  // which are appended after slot np if they stay.
  auto process = [&](bool valid, int oslot, bool incoming, int ix, int iy, float x, float y, float ux, float uy,
                     float uz) {
    // every lane runs the same instructions; invalid lanes carry a zero
    // particle and are masked out by `valid` where it matters
    int li = ix - cx0, lj = iy - cy0;
    errbits |= (valid && ((unsigned)li >= (unsigned)TX || (unsigned)lj >= (unsigned)TY)) ? ERR_ESCAPE : 0;
    li = min(max(li, 0), TX - 1);  // keeps the accesses inside the halo
    lj = min(max(lj, 0), TY - 1);
    ix = cx0 + li;
    iy = cy0 + lj;
    float mx, my, x1, y1, qvz;
    int di, dj;
    bool bad;
    const float kin = push_particle(fld, li, lj, x, y, ux, uy, uz, mx, my, x1, y1, di, dj, qvz, bad, Cl);
    if constexpr (DET) {
      long long h, l;
      efix_split(valid ? kin : 0.0f, h, l);
      khi += h;
      klo += l;
    } else {
      kahan_add(ks, kc, valid ? kin : 0.f);
    }
    errbits |= (valid && bad) ? ERR_ESCAPE : 0;
    const bool split = valid && ((di != 0) || (dj != 0));
    const bool single = valid && !split;
    // the whole motion inside the cell: one segment (particles.c:781-797);
    // crossing motions are queued below and contribute nothing here: every
    // contribution is proportional to dx, dy or qvz, so zeroing those three
    // zeroes all eight
    Seg a;
    a.x0 = x;
    a.y0 = y;
    a.dx = single ? mx : 0.f;
    a.dy = single ? my : 0.f;
    a.x1 = x + mx;
    a.y1 = y + my;
    a.qvz = single ? qvz * 0.5f : 0.f;
    a.ix = li;
    a.iy = lj;
    SegCurrent cur = segment_current(a, Cl.qnx, Cl.qny);
    const float sx0 = x, sy0 = y, smx = mx, smy = my, sqvz = qvz;
    const int spk = li | (lj << 8) | ((di + 1) << 16) | ((dj + 1) << 18);
    x = x1;
    y = y1;
    const bool keep = apply_boundary(ix, iy, di, dj, Cl);
    // (the cell is inside the grid when the particle is kept; dest is unused otherwise)
    const int dest = (int)((unsigned)ix / TX) + (int)((unsigned)iy / TY) * Cl.ntx;
    const int code = (valid && keep) ? ((dest == t) ? 1 : 2) : 0;  // 1 stays, 2 leaves

    // output, before the current sums so that the particle's registers are
    // free while they run: an own slot takes the particle back, or a hole
    if (oslot >= 0) {
      if (code == 1) store_particle(pout, base + oslot, ix, iy, x, y, ux, uy, uz);
      else store_hole(pout, base + oslot);
    }
    // leavers to the outbox, arrivals that stay appended after slot np: one
    // shared-memory atomic per warp and kind
    const unsigned mleave = __ballot_sync(0xffffffffu, code == 2);
    const unsigned mapp = incoming ? __ballot_sync(0xffffffffu, code == 1) : 0u;
    if (mleave | mapp) {
      int lb = 0, ab = 0;
      if (lane == 0) {
        if (mleave) lb = atomicAdd(&s_leave, __popc(mleave));
        if (mapp) ab = atomicAdd(&s_app, __popc(mapp));
      }
      lb = __shfl_sync(0xffffffffu, lb, 0);
      ab = __shfl_sync(0xffffffffu, ab, 0);
      if (code == 2) {
        const int s = lb + __popc(mleave & below);
        if (s < O.cap) {
          store_particle(O.p, obase + s, ix, iy, x, y, ux, uy, uz);
          O.dst[obase + s] = dest;
        } else {
          spill_particle(S, &errbits, ix, iy, x, y, ux, uy, uz);
        }
      } else if (incoming && code == 1) {
        const int s = n_own + ab + __popc(mapp & below);
        if (s < cap) store_particle(pout, base + s, ix, iy, x, y, ux, uy, uz);
        else spill_particle(S, &errbits, ix, iy, x, y, ux, uy, uz);
      }
    }

    if constexpr (DET) {
      // segmented warp reduction of the single-segment currents over runs
      // of lanes that start in the same cell (the lanes read the chunk in
      // cell order), as many halving steps as the longest run needs; each
      // lane's contributions rounded to fixed point first, then summed as
      // integers: the same total whatever lanes hold which particles
      const int key = valid ? (li + lj * TX) : -1 - lane;
      const int knext = __shfl_down_sync(0xffffffffu, key, 1);
      const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
      const unsigned lastmask = __ballot_sync(0xffffffffu, lane == 31 || knext != key);
      const int run_last = __ffs(lastmask & (0xffffffffu << lane)) - 1;
      const unsigned maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(run_last - lane + 1));
      const bool head = valid && (lane == 0 || kprev != key);
      int ih[8], im[8], il[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) jsplit(cur.v[q], Cl, ih[q], im[q], il[q]);
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        if ((unsigned)off >= maxlen) break;
        const bool take = lane + off <= run_last;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int oh = __shfl_down_sync(0xffffffffu, ih[q], off);
          const int om = __shfl_down_sync(0xffffffffu, im[q], off);
          const int ol = __shfl_down_sync(0xffffffffu, il[q], off);
          if (take) {
            ih[q] += oh;
            im[q] += om;
            il[q] += ol;
          }
        }
      }
      if (head) {
        dep.addi(0, li, lj, ih[0], im[0], il[0]);
        dep.addi(0, li, lj + 1, ih[1], im[1], il[1]);
        dep.addi(1, li, lj, ih[2], im[2], il[2]);
        dep.addi(1, li + 1, lj, ih[3], im[3], il[3]);
        dep.addi(2, li, lj, ih[4], im[4], il[4]);
        dep.addi(2, li + 1, lj, ih[5], im[5], il[5]);
        dep.addi(2, li, lj + 1, ih[6], im[6], il[6]);
        dep.addi(2, li + 1, lj + 1, ih[7], im[7], il[7]);
      }
    } else {
      // the lane's running sum: added to J when the lane's cell changes
      // (the sum is over this lane's particles of one cell, in order)
      const int key = li + lj * TX;
      const bool change = valid && key != acc_key;
      const bool flush = change && acc_key >= 0;
      if (__any_sync(0xffffffffu, flush)) {
        if (flush) add_current(dep, acc_key % TX, acc_key / TX, acc);
      }
      const float carry = change ? 0.0f : 1.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) acc.v[q] = __fmaf_rn(acc.v[q], carry, cur.v[q]);  // acc + cur, or cur
      acc_key = change ? key : acc_key;
    }

    // queue the cell-crossing motions; deposit them once QFLUSH are waiting
    {
      const unsigned sm = __ballot_sync(0xffffffffu, split);
      if (sm) {
        if (split) {
          const int e = qcount + __popc(sm & below);
          qf[warp][0][e] = sx0;
          qf[warp][1][e] = sy0;
          qf[warp][2][e] = smx;
          qf[warp][3][e] = smy;
          qf[warp][4][e] = sqvz;
          qi[warp][e] = spk;
        }
        qcount += __popc(sm);
        __syncwarp();
        if (qcount >= QFLUSH) {
          const int nq = min(qcount, 32);
          qcount -= nq;
          if (lane < nq) deposit_queued(qcount + lane);
          __syncwarp();
        }
      }
    }
  };

  // incoming particles: warp w scans the outboxes of neighbours w, w + NW,
  // ... for the slots bound for this tile and lists them; a full list
  // leaves the rest to be pushed right here
  for (int m = warp; m < nnb; m += NW) {
    const int src = nb[m];
    const int n = Oin.cnt[src];
    const long long ob = (long long)src * Oin.cap;
    for (int e0 = 0; e0 < n; e0 += 32) {
      const int e = e0 + lane;
      const bool bound = e < n && Oin.dst[ob + e] == t;
      const unsigned bm = __ballot_sync(0xffffffffu, bound);
      if (!bm) continue;
      int slot = 0;
      if (lane == 0) slot = atomicAdd(&s_nin, __popc(bm));
      slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(bm & below);
      if (bound && slot < INCAP) s_in[slot] = (e << 4) | m;
      const bool over = bound && slot >= INCAP;
      if (__any_sync(0xffffffffu, over)) {
        PRec r = {0, 0, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (over) r = load_particle(Oin.p, ob + e);
        process(over, -2, true, r.ix, r.iy, r.x, r.y, r.ux, r.uy, r.uz);
      }
    }
  }
  __syncthreads();

  // own slots: warp w takes chunks w, w + NW, ... of kChunk slots, 32 at a
  // time (a unit); its next unit is copied into shared memory while it is
  // pushed.  In a full chunk lane l of the float builds takes slot 32 k + l
  // at step k, which holds the chunk's particle l kLaneRun + k in cell
  // order; the deterministic builds take the particle 32 k + l of the cell
  // order, at its tile_slot.  Every particle goes back to the slot it came
  // from.
  {
    // read and write slots of this lane in unit u; false: no slot
    const auto slots = [&](int u, int &rs, int &ws) -> bool {
      const int c0 = (warp + NW * (u / kLaneRun)) * kChunk;
      const int k = u % kLaneRun;
      const int i = c0 + k * 32 + lane;
      if constexpr (DET) {
        if (c0 + kChunk <= n_own) {
          const int j = k * 32 + lane;
          rs = ws = c0 + (j % kLaneRun) * 32 + j / kLaneRun;
          return true;
        }
      }
      rs = ws = i;
      return i < n_own;
    };
    const auto ubase = [&](int u) { return (warp + NW * (u / kLaneRun)) * kChunk + (u % kLaneRun) * 32; };
    {
      int rs, ws;
      if (ubase(0) < n_own && slots(0, rs, ws)) {
        cp_async16(&pf_u[warp][lane], &pin.u[base + rs]);
        cp_async8(&pf_xy[warp][lane], &pin.xy[base + rs]);
      } else {
        // a lane without a first particle reads these zeros
        pf_u[warp][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
        pf_xy[warp][lane] = make_float2(0.f, 0.f);
      }
    }
    cp_async_commit();
    for (int u = 0; ubase(u) < n_own; ++u) {
      cp_async_wait<0>();  // this unit's copies (each lane its own slot) are in
      int rs, ws;
      const bool inr = slots(u, rs, ws);
      // a lane without a particle carries whatever its prefetch slot holds
      // (the last unit's particle, a hole's zero momenta, or the zeros the
      // slots start with): finite values whose results `valid` masks; its
      // position is set to the cell centre (a hole's is stale)
      const float4 uu = pf_u[warp][lane];
      const float2 xy = pf_xy[warp][lane];
      const unsigned cw = (unsigned)__float_as_int(uu.w);
      const bool valid = inr && cw != kHole;
      PRec r;
      r.ix = (int)(cw & 0xffffu);
      r.iy = (int)(cw >> 16);
      r.x = valid ? xy.x : 0.5f;
      r.y = valid ? xy.y : 0.5f;
      r.ux = uu.x;
      r.uy = uu.y;
      r.uz = uu.z;
      {
        int rn, wn;
        if (ubase(u + 1) < n_own && slots(u + 1, rn, wn)) {
          cp_async16(&pf_u[warp][lane], &pin.u[base + rn]);
          cp_async8(&pf_xy[warp][lane], &pin.xy[base + rn]);
        }
      }
      cp_async_commit();
      process(valid, inr ? ws : -2, false, r.ix, r.iy, r.x, r.y, r.ux, r.uy, r.uz);
    }
    cp_async_wait<0>();
  }

  // the listed incoming particles, in units of 32 spread over the warps
  {
    const int nin = min(s_nin, INCAP);
    for (int i = warp; i * 32 < nin; i += NW) {
      const int k = i * 32 + lane;
      const bool valid = k < nin;
      PRec r = {0, 0, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (valid) {
        const int v = s_in[k];
        r = load_particle(Oin.p, (long long)nb[v & 15] * Oin.cap + (v >> 4));
      }
      process(valid, -2, true, r.ix, r.iy, r.x, r.y, r.ux, r.uy, r.uz);
    }
  }

  if (lane < qcount) deposit_queued(lane);  // what is left in the queue
  if constexpr (!DET)
    if (acc_key >= 0) add_current(dep, acc_key % TX, acc_key / TX, acc);  // the lanes' last sums

  __syncthreads();
  if (threadIdx.x == 0) {
    T.np[t] = n_own + min(s_app, cap - n_own);
    O.cnt[t] = min(s_leave, O.cap);
  }
  if constexpr (DET) {
    // integer sums: exact in any order
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      khi += __shfl_down_sync(0xffffffffu, khi, off);
      klo += __shfl_down_sync(0xffffffffu, klo, off);
    }
    if (lane == 0) {
      if (khi) atomicAdd(&s_ekin[0], (unsigned long long)khi);
      if (klo) atomicAdd(&s_ekin[1], (unsigned long long)klo);
    }
    __syncthreads();
    if (threadIdx.x == 0) ekin_tile[t] = efix_join((long long)s_ekin[0], (long long)s_ekin[1]);
    // the integer J tile goes to the global fixed-point planes (units of
    // 2^-40) with 64-bit integer atomics (cells outside the buffer hold no
    // deposits)
    for (int k = threadIdx.x; k < LAY::N; k += NT) {
      const long long v = tile_node_sum(sJi, LAY::N, k, Cl.js_l);
      if (!v) continue;
      int c, r, col;
      LAY::where(k, c, r, col);
      const int gy = cy0 + r, gx = cx0 + col;
      if (gx < fj.pitch && (size_t)gy * fj.pitch < fj.plane)
        atomicAdd(&fj.p[c * fj.plane + (size_t)gy * fj.pitch + gx], (unsigned long long)(v * Cl.js_det));
    }
    if (threadIdx.x == 0 && !loaded && !mbar_wait_bounded(&bar, 0))
      errbits |= ERR_TIMEOUT;  // second bounded wait for the load still in flight
  } else {
    const double e = block_sum_double<NT>((double)ks - (double)kc, sred);
    if (threadIdx.x == 0) ekin_tile[t] = e;

    if (threadIdx.x == 0 && !loaded && !mbar_wait_bounded(&bar, 0))
      errbits |= ERR_TIMEOUT;  // second bounded wait for the load still in flight
  }
  if (errbits) atomicOr(err, errbits);
}

// ---------------------------------------------------------------------------
// spill push: same physics from global memory (rarely non-empty)
// ---------------------------------------------------------------------------
template <int NT, bool DET>
__global__ void __launch_bounds__(NT) k_push_spill(const float *EB, float *J, FixedJ fj, Grid G, Particles sin,
                                                   const int *sin_cnt, int sin_cap, Spill S, double *ekin,
                                                   int *err, PushConst C) {
  __shared__ double sred[NT / 32];
  const int n = min(*sin_cnt, sin_cap);
  if (n == 0) return;  // the usual case: nothing spilled (uniform across the grid)
  const GlobalFields fld{EB, G.pitch, G.plane};
  const auto dep = [&] {
    if constexpr (DET)
      return GlobalCurrentFixed{fj.p, fj.pitch, fj.plane, &C};
    else
      return GlobalCurrent{J, G.pitch, G.plane};
  }();
  int errbits = 0;
  float ks = 0.f, kc = 0.f;
  long long khi = 0, klo = 0;
  for (int k = blockIdx.x * NT + threadIdx.x; k < n; k += gridDim.x * NT) {
    const PRec r = load_particle(sin, k);
    int ix = r.ix, iy = r.iy;
    float x = r.x, y = r.y, ux = r.ux, uy = r.uy, uz = r.uz;
    if (ix < 0 || ix >= C.nx || iy < 0 || iy >= C.ny) {
      errbits |= ERR_ESCAPE;
      ix = min(max(ix, 0), C.nx - 1);
      iy = min(max(iy, 0), C.ny - 1);
    }
    float mx, my, x1, y1, qvz;
    int di, dj;
    bool bad;
    const float kin = push_particle(fld, ix, iy, x, y, ux, uy, uz, mx, my, x1, y1, di, dj, qvz, bad, C);
    if (bad) errbits |= ERR_ESCAPE;
    if constexpr (DET) {
      long long h, l;
      efix_split(kin, h, l);
      khi += h;
      klo += l;
    } else {
      kahan_add(ks, kc, kin);
    }
    const Seg a = zigzag_first(dep, ix, iy, di, dj, x, y, mx, my, C.qnx, C.qny, qvz);
    add_current(dep, ix, iy, segment_current(a, C.qnx, C.qny));
    x = x1;
    y = y1;
    if (apply_boundary(ix, iy, di, dj, C)) spill_particle(S, &errbits, ix, iy, x, y, ux, uy, uz);
  }
  if constexpr (DET) {
    if (khi) atomicAdd(reinterpret_cast<unsigned long long *>(ekin), (unsigned long long)khi);
    if (klo) atomicAdd(reinterpret_cast<unsigned long long *>(ekin) + 1, (unsigned long long)klo);
  } else {
    const double e = block_sum_double<NT>((double)ks - (double)kc, sred);
    if (threadIdx.x == 0 && e != 0.0) atomicAdd(ekin, e);
  }
  if (errbits) atomicOr(err, errbits);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <int TX, int TY, bool DET>
static cudaError_t launch_push_t(const PushLaunch &a, cudaStream_t st) {
  // 4 warps per CTA (8 CTAs per SM: shorter barriers, CTAs in more phases);
  // the deterministic build's integer J tile keeps 8 warps per CTA
  constexpr int NT = (DET && TX * TY >= 256) ? 256 : 128;
  k_push_tiles<TX, TY, NT, DET><<<a.ntiles, NT, 0, st>>>(*a.tm_eb, a.pin, a.pout, a.T, a.Oin, a.O, a.S,
                                                           a.ekin_tile, a.err, a.C, a.fj);
  return cudaGetLastError();
}

// nothing to prepare: every variant runs with static shared memory only
template <int TX, int TY, bool DET>
static cudaError_t prepare_push_t() {
  return cudaSuccess;
}

template <bool DET>
static cudaError_t prepare_push_variant(int TX, int TY) {
#define ZC_TILE(X, Y) \
  if (TX == X && TY == Y) return prepare_push_t<X, Y, DET>();
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

template <bool DET>
static cudaError_t launch_push_tiles_variant(const PushLaunch &a, cudaStream_t st) {
  const int TX = a.TX, TY = a.TY;
#define ZC_TILE(X, Y) \
  if (TX == X && TY == Y) return launch_push_t<X, Y, DET>(a, st);
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

template <bool DET>
static cudaError_t launch_push_spill_variant(const float *EB, float *J, const FixedJ &fj, const Grid &G,
                                             const Particles &sin, const int *sin_cnt, int sin_cap, const Spill &S,
                                             double *ekin, int *err, const PushConst &C, int nblocks,
                                             cudaStream_t st) {
  k_push_spill<256, DET><<<nblocks, 256, 0, st>>>(EB, J, fj, G, sin, sin_cnt, sin_cap, S, ekin, err, C);
  return cudaGetLastError();
}
