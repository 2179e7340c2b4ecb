// zc_em1d.cu -- the em1d step on the GPU (libzpic_cuda, C-ABI zc1_*).
//
// Restates the reference's em1d time step (em1d/simulation.c:45-56):
// current_zero; per species the push -- gather (interpolate_fld,
// em1d/particles.c:864-894), relativistic Boris, move, 1-D zigzag deposit
// (dep_current_zamb, particles.c:707-790), window shift + cold injection and
// absorbing / periodic boundaries (particles.c:1040-1062, 594-612); then
// current_update (guard fold + binomial / compensated passes,
// em1d/current.c:111-330) and emf_advance (yee_b, yee_e, Mur, yee_b, guard
// cells, window shift, em1d/emf.c:379-580).
//
// Layout: particles are SoA arrays (ix, x, ux, uy, uz) on the device, kept
// in cell order by a counting sort every few steps so that the lanes of a
// warp share cells; E, B, J are the reference's float3 buffers (one lower and
// two upper guard cells).  The push runs one particle per lane: the current
// of a motion that stays in its cell is summed over the lanes of the cell
// (segmented warp reduction) and added to J with one float reduction per
// node (performed in L2); cell-crossing motions add their two segments
// directly.  1-D grids are small, so the field and current phases run in
// one CTA each.  Compiled with --fmad=false: every float operation rounds as
// in the reference C, so particles advanced from the same fields land on the
// same bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <new>
#include <vector>

#include "../../include/zpic_cuda.h"
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace zc1 {

constexpr int GC0 = 1, GC1 = 2;  // guard cells (em1d/emf.c:59)
constexpr int kDead = -(1 << 30);
enum { ERR1_ESCAPE = 1, ERR1_OVERFLOW = 2 };

struct Parts {
  int *ix;
  float *x, *ux, *uy, *uz;
};

struct Push1 {
  float tem, dt_dx, qnx, q;
  int nx;
  int shift;  // window shift this step (0/1)
  int open;   // absorb particles leaving [0, nx)
};

__device__ __forceinline__ float lerp1(const float *F, int i, int c, float w) {
  return F[(i + GC0) * 3 + c] * (1.0f - w) + F[(i + 1 + GC0) * 3 + c] * w;
}

__device__ __forceinline__ void red(float *J, int i, int c, float v) { atomicAdd(&J[(i + GC0) * 3 + c], v); }

// the five contributions of one segment inside cell ix (particles.c:770-788):
// Jx at ix, Jy and Jz at ix and ix+1
struct Seg1 {
  float jx, y0, y1, z0, z1;
};

__device__ __forceinline__ Seg1 seg_current(float x0, float x1, float dx, float qvy, float qvz, float qnx) {
  const float s00 = 1.0f - x0, s01 = x0;
  const float s10 = 1.0f - x1, s11 = x1;
  Seg1 r;
  r.jx = qnx * dx;
  r.y0 = qvy * (s00 + s10 + (s00 - s10) / 2.0f);
  r.y1 = qvy * (s01 + s11 + (s01 - s11) / 2.0f);
  r.z0 = qvz * (s00 + s10 + (s00 - s10) / 2.0f);
  r.z1 = qvz * (s01 + s11 + (s01 - s11) / 2.0f);
  return r;
}

__device__ __forceinline__ void add_seg(float *J, int ix, const Seg1 &s) {
  red(J, ix, 0, s.jx);
  red(J, ix, 1, s.y0);
  red(J, ix + 1, 1, s.y1);
  red(J, ix, 2, s.z0);
  red(J, ix + 1, 2, s.z1);
}

// ---------------------------------------------------------------------------
// push + deposit, one particle per lane, warps over consecutive particles
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k1_push(Parts p, const int *d_np, const float *E, const float *B, float *J,
                                               Push1 C, double *ekin, int *err) {
  __shared__ double sred[8];
  const int n = *d_np;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  float ks = 0.f, kc = 0.f;
  int errbits = 0;
  for (int base = gw * 32; base < n; base += nw * 32) {
    const int i = base + lane;
    const bool valid = i < n;
    int ix = 0;
    float x = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
    if (valid) {
      ix = p.ix[i];
      x = p.x[i];
      ux = p.ux[i];
      uy = p.uy[i];
      uz = p.uz[i];
      if (ix < 0 || ix >= C.nx) {
        errbits |= ERR1_ESCAPE;
        ix = min(max(ix, 0), C.nx - 1);
      }
    }
    // staggered linear gather (particles.c:864-894)
    const int ih = ix + ((x < 0.5f) ? -1 : 0);
    const float w1h = x + ((x < 0.5f) ? 0.5f : -0.5f);
    float ex = lerp1(E, ih, 0, w1h), ey = lerp1(E, ix, 1, x), ez = lerp1(E, ix, 2, x);
    float bx = lerp1(B, ix, 0, x), by = lerp1(B, ih, 1, w1h), bz = lerp1(B, ih, 2, w1h);
    // Boris (particles.c:960-1010)
    ex *= C.tem;
    ey *= C.tem;
    ez *= C.tem;
    float utx = ux + ex, uty = uy + ey, utz = uz + ez;
    const float u2 = utx * utx + uty * uty + utz * utz;
    const float gamma = sqrtf(1 + u2);
    const float kin = u2 / (1 + gamma);
    const float gtem = C.tem / gamma;
    bx *= gtem;
    by *= gtem;
    bz *= gtem;
    const float otsq = 2.0f / (1.0f + bx * bx + by * by + bz * bz);
    ux = utx + uty * bz - utz * by;
    uy = uty + utz * bx - utx * bz;
    uz = utz + utx * by - uty * bx;
    bx *= otsq;
    by *= otsq;
    bz *= otsq;
    utx += uy * bz - uz * by;
    uty += uz * bx - ux * bz;
    utz += ux * by - uy * bx;
    ux = utx + ex;
    uy = uty + ey;
    uz = utz + ez;
    // move (particles.c:1012-1022)
    const float rg = 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
    const float dx = C.dt_dx * rg * ux;
    float x1 = x + dx;
    const int di = (x1 >= 1.0f) - (x1 < 0.0f);
    x1 -= di;
    const float qvy = C.q * uy * rg;
    const float qvz = C.q * uz * rg;
    if (valid) {
      const float y = kin - kc;
      const float t = ks + y;
      kc = (t - ks) - y;
      ks = t;
      if (!(fabsf(dx) < 1.0f)) errbits |= ERR1_ESCAPE;
    }
    // deposit (dep_current_zamb): qvy, qvz halved, split at the cell edge
    const float hy = qvy / 2.0f, hz = qvz / 2.0f;
    const bool split = valid && di != 0;
    Seg1 s = seg_current(x, x + dx, dx, hy, hz, C.qnx);
    if (split) {
      const int ib = (di == 1);
      const float delta = (x + dx - ib) / dx;
      const Seg1 b = seg_current(1 - ib, (x + dx) - di, dx * delta, hy * delta, hz * delta, C.qnx);
      add_seg(J, ix + di, b);
      s = seg_current(x, (float)ib, dx * (1.0f - delta), hy * (1.0f - delta), hz * (1.0f - delta), C.qnx);
      add_seg(J, ix, s);
    }
    // single-segment motions: summed over the lanes of a cell, one lane
    // per cell adds them (the lanes of a run are contiguous in cell order)
    {
      const bool single = valid && !split;
      const int key = single ? ix : -1 - lane;
      const int knext = __shfl_down_sync(0xffffffffu, key, 1);
      const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
      const unsigned lastmask = __ballot_sync(0xffffffffu, lane == 31 || knext != key);
      const int run_last = __ffs(lastmask & (0xffffffffu << lane)) - 1;
      const unsigned maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(run_last - lane + 1));
      const bool head = single && (lane == 0 || kprev != key);
      float v[5] = {single ? s.jx : 0.f, single ? s.y0 : 0.f, single ? s.y1 : 0.f, single ? s.z0 : 0.f,
                    single ? s.z1 : 0.f};
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        if ((unsigned)off >= maxlen) break;
        const bool take = lane + off <= run_last;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          const float o = __shfl_down_sync(0xffffffffu, v[q], off);
          if (take) v[q] += o;
        }
      }
      if (head) add_seg(J, ix, Seg1{v[0], v[1], v[2], v[3], v[4]});
    }
    // boundaries (particles.c:1040-1062)
    if (valid) {
      int nix = ix + di - C.shift;
      if (C.open) {
        if (nix < 0 || nix >= C.nx) nix = kDead;
      } else {
        nix += ((nix < 0) ? C.nx : 0) - ((nix >= C.nx) ? C.nx : 0);
      }
      p.ix[i] = nix;
      p.x[i] = x1;
      p.ux[i] = ux;
      p.uy[i] = uy;
      p.uz[i] = uz;
    }
  }
  const double e = zc::block_sum_double<256>((double)ks - (double)kc, sred);
  if (threadIdx.x == 0 && e != 0.0) atomicAdd(ekin, e);
  if (errbits) atomicOr(err, errbits);
}

// ---------------------------------------------------------------------------
// order-preserving compaction of the live particles (open boundaries,
// moving window): counts per block, one-block scan, scatter
// ---------------------------------------------------------------------------
constexpr int kCompactBlock = 256;
constexpr int kCompactPer = 2048;  // particles per block

__global__ void k1_live_count(const int *ix, const int *d_np, int *blk) {
  __shared__ int sw[kCompactBlock / 32];
  const int n = *d_np;
  const int b0 = blockIdx.x * kCompactPer;
  int c = 0;
  for (int i = b0 + threadIdx.x; i < min(n, b0 + kCompactPer); i += kCompactBlock) c += (ix[i] != kDead);
  int tot;
  zc::block_exclusive_scan<kCompactBlock>(c, tot, sw);
  if (threadIdx.x == 0) blk[blockIdx.x] = tot;
}

__global__ void k1_scan_blocks(int *blk, int nblk, int *d_np) {
  __shared__ int sw[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nblk; b0 += 1024) {
    const int v = (b0 + (int)threadIdx.x < nblk) ? blk[b0 + threadIdx.x] : 0;
    int tot;
    const int pre = zc::block_exclusive_scan<1024>(v, tot, sw);
    if (b0 + (int)threadIdx.x < nblk) blk[b0 + threadIdx.x] = carry + pre;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *d_np = carry;
}

__global__ void k1_live_scatter(Parts src, Parts dst, const int *d_np_old, const int *blk) {
  __shared__ int sw[kCompactBlock / 32];
  __shared__ int sbase;
  const int n = *d_np_old;
  const int b0 = blockIdx.x * kCompactPer;
  if (threadIdx.x == 0) sbase = blk[blockIdx.x];
  __syncthreads();
  for (int c0 = b0; c0 < min(n, b0 + kCompactPer); c0 += kCompactBlock) {
    const int i = c0 + threadIdx.x;
    const bool live = i < n && src.ix[i] != kDead;
    int tot;
    const int pre = zc::block_exclusive_scan<kCompactBlock>(live ? 1 : 0, tot, sw);
    if (live) {
      const int o = sbase + pre;
      dst.ix[o] = src.ix[i];
      dst.x[o] = src.x[i];
      dst.ux[o] = src.ux[i];
      dst.uy[o] = src.uy[i];
      dst.uz[o] = src.uz[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) sbase += tot;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// cold injection of the column nx-1 after a window move (spec_set_x for
// uniform / step / slab profiles, particles.c:250-300; momenta = ufl, the
// thermal part being zero)
// ---------------------------------------------------------------------------
struct Inject1 {
  int ppc, type;  // density type: 0 uniform, 1 empty, 2 step, 3 slab
  float start, end, dx;
  float ufl[3];
};

__global__ void k1_inject(Parts p, int *d_np, int cap, Inject1 I, int nx, int n_move, int *err) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (I.type == 1) return;
  int n = *d_np;
  const int i = nx - 1;
  const float start = I.start / I.dx - n_move;
  const float end = I.end / I.dx - n_move;
  for (int k = 0; k < I.ppc; ++k) {
    const float pos = (float)((k + 0.5) / I.ppc);
    bool take = true;
    if (I.type == 2) take = i + pos > start;
    if (I.type == 3) take = i + pos > start && i + pos < end;
    if (!take) continue;
    if (n >= cap) {
      atomicOr(err, ERR1_OVERFLOW);
      break;
    }
    p.ix[n] = i;
    p.x[n] = pos;
    p.ux[n] = I.ufl[0];
    p.uy[n] = I.ufl[1];
    p.uz[n] = I.ufl[2];
    ++n;
  }
  *d_np = n;
}

// ---------------------------------------------------------------------------
// counting sort by cell (src -> dst); counts and cursors over nx cells,
// warp-aggregated atomics (the input is mostly sorted already)
// ---------------------------------------------------------------------------
__global__ void k1_cell_count(const int *ix, const int *d_np, int *cnt) {
  const int n = *d_np;
  for (int b = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b < n; b += gridDim.x * blockDim.x) {
    const int i = b + (threadIdx.x & 31);
    const int key = i < n ? ix[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (i < n && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[key], __popc(peers));
  }
}

__global__ void k1_cell_scan(int *cnt, int nx) {
  __shared__ int sw[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nx; b0 += 1024) {
    const int v = (b0 + (int)threadIdx.x < nx) ? cnt[b0 + threadIdx.x] : 0;
    int tot;
    const int pre = zc::block_exclusive_scan<1024>(v, tot, sw);
    if (b0 + (int)threadIdx.x < nx) cnt[b0 + threadIdx.x] = carry + pre;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

__global__ void k1_cell_scatter(Parts src, Parts dst, const int *d_np, int *cursor) {
  const int n = *d_np;
  const int lane = threadIdx.x & 31;
  for (int b = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b < n; b += gridDim.x * blockDim.x) {
    const int i = b + lane;
    const int key = i < n ? src.ix[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (i < n && lane == leader) base = atomicAdd(&cursor[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (i < n) {
      const int o = base + __popc(peers & ((1u << lane) - 1));
      dst.ix[o] = key;
      dst.x[o] = src.x[i];
      dst.ux[o] = src.ux[i];
      dst.uy[o] = src.uy[i];
      dst.uz[o] = src.uz[i];
    }
  }
}

// ---------------------------------------------------------------------------
// current update (current.c:111-330): periodic guard fold, then the filter
// passes, each out of place into the other buffer; one CTA
// ---------------------------------------------------------------------------
struct Smooth1 {
  int n;
  float sa[16], sb[16];
};

__global__ void __launch_bounds__(1024) k1_current(float *J0, float *J1, int nx, int periodic, Smooth1 S,
                                                  int *which) {
  float *J = J0, *O = J1;
  if (periodic) {
    // J[i] += J[nx + i] for i = -1, 0, 1, then the upper cells copy the lower
    if (threadIdx.x < 9) {
      const int i = (int)threadIdx.x / 3 - 1, c = threadIdx.x % 3;
      J[(i + GC0) * 3 + c] += J[(nx + i + GC0) * 3 + c];
    }
    __syncthreads();
    if (threadIdx.x < 9) {
      const int i = (int)threadIdx.x / 3 - 1, c = threadIdx.x % 3;
      J[(nx + i + GC0) * 3 + c] = J[(i + GC0) * 3 + c];
    }
    __syncthreads();
  }
  for (int p = 0; p < S.n; ++p) {
    const float sa = S.sa[p], sb = S.sb[p];
    for (int k = threadIdx.x; k < nx * 3; k += blockDim.x) {
      const int i = k / 3, c = k % 3;
      O[(i + GC0) * 3 + c] =
          sa * J[(i - 1 + GC0) * 3 + c] + sb * J[(i + GC0) * 3 + c] + sa * J[(i + 1 + GC0) * 3 + c];
    }
    __syncthreads();
    // guard cells: periodic copies of the filtered cells, else as they were
    if (threadIdx.x < 9) {
      const int g = threadIdx.x / 3, c = threadIdx.x % 3;  // g: guard -1, nx, nx+1
      const int gi = (g == 0) ? -1 : nx + g - 1;
      const int src = (g == 0) ? nx - 1 : g - 1;
      O[(gi + GC0) * 3 + c] = periodic ? O[(src + GC0) * 3 + c] : J[(gi + GC0) * 3 + c];
    }
    __syncthreads();
    float *t = J;
    J = O;
    O = t;
  }
  if (threadIdx.x == 0) *which = (J == J0) ? 0 : 1;
}

// ---------------------------------------------------------------------------
// field advance (emf.c:379-580), one CTA: yee_b(dt/2), yee_e(dt), Mur,
// yee_b(dt/2), guard cells, window shift
// ---------------------------------------------------------------------------
struct Emf1 {
  int nx;
  float dt, dx;
  int bc;  // 0 none, 1 periodic, 2 open (Mur)
  int shift;
};

__device__ __forceinline__ void yee_b1(float *E, float *B, int nx, float dt_dx) {
  for (int i = (int)threadIdx.x - 1; i <= nx; i += blockDim.x) {
    const int k = (i + GC0) * 3;
    B[k + 1] += (dt_dx * (E[k + 3 + 2] - E[k + 2]));
    B[k + 2] += (-dt_dx * (E[k + 3 + 1] - E[k + 1]));
  }
}

// periodic guard cells of E and B (emf_update_gc, emf.c:476-500): -1 <- nx-1
// and nx <- 0 only; the second upper guard cell nx+1 keeps the value yee_e
// gave it.  Threads 0..11 of the CTA.
__device__ __forceinline__ void periodic_gc1(float *E, float *B, int nx) {
  if (threadIdx.x < 12) {
    float *F = (threadIdx.x < 6) ? E : B;
    const int t = threadIdx.x % 6, g = t / 3, c = t % 3;
    const int gi = (g == 0) ? -1 : nx;
    const int src = (g == 0) ? nx - 1 : 0;
    F[(gi + GC0) * 3 + c] = F[(src + GC0) * 3 + c];
  }
}

__global__ void __launch_bounds__(1024) k1_emf(float *E, float *B, const float *J, float *mur, Emf1 M) {
  const int nx = M.nx;
  const float hdt = M.dt / 2.0f;
  yee_b1(E, B, nx, hdt / M.dx);
  __syncthreads();
  {
    const float dt_dx = M.dt / M.dx, dt = M.dt;
    for (int i = threadIdx.x; i <= nx + 1; i += blockDim.x) {
      const int k = (i + GC0) * 3;
      E[k + 0] += (-dt * J[k + 0]);
      E[k + 1] += (-dt_dx * (B[k + 2] - B[k - 3 + 2]) - dt * J[k + 1]);
      E[k + 2] += (+dt_dx * (B[k + 1] - B[k - 3 + 1]) - dt * J[k + 2]);
    }
  }
  __syncthreads();
  if (M.bc == 2 && threadIdx.x == 0) {
    // first-order Mur (emf.c:379-415); mur = fld[2][3], tmp[2][3]
    float *fld = mur, *tmp = mur + 6;
    const float S = (M.dt - M.dx) / (M.dt + M.dx);
    const int lo = (0 + GC0) * 3, hi = (nx - 1 + GC0) * 3;
    fld[1] = tmp[1] + S * (E[lo + 1] - fld[1]);
    fld[2] = tmp[2] + S * (E[lo + 2] - fld[2]);
    E[(-1 + GC0) * 3 + 1] = fld[1];
    E[(-1 + GC0) * 3 + 2] = fld[2];
    tmp[1] = E[lo + 1];
    tmp[2] = E[lo + 2];
    fld[4] = tmp[4] + S * (E[hi + 1] - fld[4]);
    fld[5] = tmp[5] + S * (E[hi + 2] - fld[5]);
    E[(nx + GC0) * 3 + 1] = fld[4];
    E[(nx + GC0) * 3 + 2] = fld[5];
    tmp[4] = E[hi + 1];
    tmp[5] = E[hi + 2];
  }
  __syncthreads();
  yee_b1(E, B, nx, hdt / M.dx);
  __syncthreads();
  if (M.bc == 1) periodic_gc1(E, B, nx);
  if (M.shift) {
    // shift left one cell, zero the cells nx-1 .. nx+1 (emf.c:513-540)
    __syncthreads();
    const int ncell = nx + GC0 + GC1;
    for (int base = 0; base < ncell * 3; base += blockDim.x) {
      // buffer index k <- k + 3 for k < (ncell - 1) * 3, read before any write
      const int k = base + threadIdx.x;
      float ve = 0.f, vb = 0.f;
      if (k < (ncell - 1) * 3) {
        ve = E[k + 3];
        vb = B[k + 3];
      }
      __syncthreads();
      if (k < (ncell - 1) * 3) {
        E[k] = ve;
        B[k] = vb;
      }
      __syncthreads();
    }
    for (int k = (nx - 1 + GC0) * 3 + threadIdx.x; k < ncell * 3; k += blockDim.x) {
      E[k] = 0.f;
      B[k] = 0.f;
    }
  }
}

// laser launch (emf_add_laser, em1d/emf.c:191-260): the plane-wave pulse
// added to Ey/Ez at the cell nodes and By/Bz half a cell ahead, with the
// reference's float/double mix; periodic runs then refresh the guard cells
__global__ void __launch_bounds__(1024) k1_laser(float *E, float *B, int nx, zc::LaserConst L, int periodic) {
  const float amp = L.omega0 * L.a0;
  const float cp = cos((double)L.polarization), sp = sin((double)L.polarization);
  const float k = L.omega0;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const float z = i * L.dx, z2 = z + L.dx / 2;
    const float a = amp * zc::laser_env(L, z), a2 = amp * zc::laser_env(L, z2);
    const int o = (i + GC0) * 3;
    E[o + 1] += +a * cos((double)(k * z)) * cp;
    E[o + 2] += +a * cos((double)(k * z)) * sp;
    B[o + 1] += -a2 * cos((double)(k * z2)) * sp;
    B[o + 2] += +a2 * cos((double)(k * z2)) * cp;
  }
  __syncthreads();
  if (periodic) periodic_gc1(E, B, nx);
}

// field energy per component (emf.c:590-612): double sums of float squares
__global__ void __launch_bounds__(1024) k1_emf_energy(const float *E, const float *B, int nx, float dx, double *out) {
  __shared__ double sred[32];
  for (int c = 0; c < 6; ++c) {
    const float *F = (c < 3) ? E : B;
    double s = 0.0;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
      const float v = F[(i + GC0) * 3 + c % 3];
      s += (double)(v * v);
    }
    const double t = zc::block_sum_double<1024>(s, sred);
    if (threadIdx.x == 0) out[c] = t * (0.5 * dx);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Species1 {
  float m_q, q;
  Inject1 inj;
  int iter = 0, n_move = 0;
  int cap = 0;
  int np_bound = 0;  // upper bound of the device count (injections since the last read)
  Parts buf[2] = {};
  int cur = 0;
  int *d_np = nullptr;
  double *d_ekin = nullptr;
  double ekin = 0.0;
};

}  // namespace zc1

using namespace zc1;

struct zc1_sim {
  int nx;
  float box, dx, dt;
  int device;
  int field_bc, current_periodic, part_open, mw, sort_every;
  int iter = 0, n_move = 0;
  Smooth1 smooth{};
  cudaStream_t st = nullptr;
  float *E = nullptr, *B = nullptr, *J[2] = {nullptr, nullptr}, *mur = nullptr;
  int j_cur = 0;
  int *d_which = nullptr, *d_err = nullptr, *d_blk = nullptr, *d_cnt = nullptr;
  int blk_cap = 0;
  double *d_emf = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  long long launches = 0;  // kernels launched by the step so far
  // optional per-kernel timing: an event pair around every launch, summed
  // per kind after the steps (zc1_set_profile / zc1_get_profile)
  int profile = 0;
  std::vector<cudaEvent_t> prof_ev;
  std::vector<int> prof_kind;
  size_t prof_used = 0;
  double prof_ms[ZC1_NKIND] = {};
  long long prof_n[ZC1_NKIND] = {};
  std::vector<Species1> sp;
};

namespace {

zc_status fail1f(zc_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  zc::set_error_message(buf);
  return s;
}

zc_status fail1(zc_status s, const char *what) { return fail1f(s, "%s", what); }

#define CK1(call)                                                                               \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return fail1f(ZC_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));    \
  } while (0)
#define TRY1(call)                \
  do {                            \
    zc_status r_ = (call);        \
    if (r_ != ZC_OK) return r_;   \
  } while (0)

struct Guard1 {
  int old = 0;
  explicit Guard1(int d) {
    cudaGetDevice(&old);
    cudaSetDevice(d);
  }
  ~Guard1() { cudaSetDevice(old); }
};

int grid_blocks() { return 152 * 8; }

zc_status alloc_parts(Parts &p, int cap) {
  CK1(cudaMalloc(&p.ix, sizeof(int) * (size_t)std::max(cap, 1)));
  CK1(cudaMalloc(&p.x, sizeof(float) * (size_t)std::max(cap, 1)));
  CK1(cudaMalloc(&p.ux, sizeof(float) * (size_t)std::max(cap, 1)));
  CK1(cudaMalloc(&p.uy, sizeof(float) * (size_t)std::max(cap, 1)));
  CK1(cudaMalloc(&p.uz, sizeof(float) * (size_t)std::max(cap, 1)));
  return ZC_OK;
}

void free_parts(Parts &p) {
  cudaFree(p.ix);
  cudaFree(p.x);
  cudaFree(p.ux);
  cudaFree(p.uy);
  cudaFree(p.uz);
  p = Parts{};
}

zc_status copy_parts(const Parts &src, const Parts &dst, int n, cudaStream_t st) {
  if (n <= 0) return ZC_OK;
  CK1(cudaMemcpyAsync(dst.ix, src.ix, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
  CK1(cudaMemcpyAsync(dst.x, src.x, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  CK1(cudaMemcpyAsync(dst.ux, src.ux, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  CK1(cudaMemcpyAsync(dst.uy, src.uy, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  CK1(cudaMemcpyAsync(dst.uz, src.uz, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  return ZC_OK;
}

int read_np(zc1_sim *s, Species1 &p) {
  int n = 0;
  cudaMemcpyAsync(&n, p.d_np, sizeof(int), cudaMemcpyDeviceToHost, s->st);
  cudaStreamSynchronize(s->st);
  p.np_bound = n;
  return n;
}

// room for `extra` more particles in both buffers, keeping the current ones;
// the device count is read (a sync) only when its upper bound no longer fits,
// and the buffers grow only when the true count does not
zc_status ensure_cap(zc1_sim *s, Species1 &p, int extra) {
  if (p.np_bound + extra <= p.cap) return ZC_OK;
  const int n = read_np(s, p);
  const int need = n + extra;
  if (need <= p.cap) return ZC_OK;
  const int cap = std::max(need, (int)(1.25 * n) + 1024);
  Parts nb[2];
  for (int b = 0; b < 2; ++b) {
    zc_status r = alloc_parts(nb[b], cap);
    if (r != ZC_OK) return r;
  }
  zc_status r = copy_parts(p.buf[p.cur], nb[0], n, s->st);
  if (r != ZC_OK) return r;
  CK1(cudaStreamSynchronize(s->st));
  free_parts(p.buf[0]);
  free_parts(p.buf[1]);
  p.buf[0] = nb[0];
  p.buf[1] = nb[1];
  p.cur = 0;
  p.cap = cap;
  return ZC_OK;
}

zc_status check_err(zc1_sim *s) {
  int e = 0;
  CK1(cudaMemcpyAsync(&e, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK1(cudaStreamSynchronize(s->st));
  if (e & ERR1_OVERFLOW) return fail1(ZC_EOVERFLOW, "1-D particle buffer full at injection");
  if (e & ERR1_ESCAPE) return fail1(ZC_EPARTICLE_ESCAPE, "a particle moved a cell or more, or left the grid");
  return ZC_OK;
}

// start of a profiled launch of `kind`: returns the slot of its event pair
// (-1 when profiling is off)
int prof_begin(zc1_sim *s, int kind) {
  if (!s->profile) return -1;
  const size_t slot = s->prof_used;
  if (2 * slot + 2 > s->prof_ev.size()) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      if (a) cudaEventDestroy(a);
      return -1;
    }
    s->prof_ev.push_back(a);
    s->prof_ev.push_back(b);
    s->prof_kind.push_back(kind);
  }
  s->prof_kind[slot] = kind;
  cudaEventRecord(s->prof_ev[2 * slot], s->st);
  s->prof_used = slot + 1;
  return (int)slot;
}

void prof_end(zc1_sim *s, int slot) {
  if (slot >= 0) cudaEventRecord(s->prof_ev[2 * (size_t)slot + 1], s->st);
}

// adds the recorded launches to the per-kind sums (after a stream sync)
void prof_collect(zc1_sim *s) {
  for (size_t i = 0; i < s->prof_used; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s->prof_ev[2 * i], s->prof_ev[2 * i + 1]) == cudaSuccess) {
      s->prof_ms[s->prof_kind[i]] += ms;
      s->prof_n[s->prof_kind[i]] += 1;
    }
  }
  s->prof_used = 0;
}

zc_status compact(zc1_sim *s, Species1 &p) {
  const int nblk = (p.np_bound + kCompactPer - 1) / kCompactPer;
  if (nblk == 0) return ZC_OK;
  if (nblk > s->blk_cap) {
    cudaFree(s->d_blk);
    s->d_blk = nullptr;
    CK1(cudaMalloc(&s->d_blk, sizeof(int) * (size_t)nblk * 2));
    s->blk_cap = nblk;
  }
  int *d_old = s->d_blk + nblk;  // the count before compaction
  CK1(cudaMemcpyAsync(d_old, p.d_np, sizeof(int), cudaMemcpyDeviceToDevice, s->st));
  const int pf = prof_begin(s, ZC1_K_COMPACT);
  k1_live_count<<<nblk, kCompactBlock, 0, s->st>>>(p.buf[p.cur].ix, d_old, s->d_blk);
  k1_scan_blocks<<<1, 1024, 0, s->st>>>(s->d_blk, nblk, p.d_np);
  k1_live_scatter<<<nblk, kCompactBlock, 0, s->st>>>(p.buf[p.cur], p.buf[1 - p.cur], d_old, s->d_blk);
  prof_end(s, pf);
  CK1(cudaGetLastError());
  s->launches += 3;
  p.cur = 1 - p.cur;
  return ZC_OK;
}

zc_status sort_cells(zc1_sim *s, Species1 &p) {
  const int pf = prof_begin(s, ZC1_K_SORT);
  CK1(cudaMemsetAsync(s->d_cnt, 0, sizeof(int) * s->nx, s->st));
  k1_cell_count<<<grid_blocks(), 256, 0, s->st>>>(p.buf[p.cur].ix, p.d_np, s->d_cnt);
  k1_cell_scan<<<1, 1024, 0, s->st>>>(s->d_cnt, s->nx);
  k1_cell_scatter<<<grid_blocks(), 256, 0, s->st>>>(p.buf[p.cur], p.buf[1 - p.cur], p.d_np, s->d_cnt);
  prof_end(s, pf);
  CK1(cudaGetLastError());
  s->launches += 3;
  p.cur = 1 - p.cur;
  return ZC_OK;
}

zc_status step1(zc1_sim *s) {
  cudaStream_t st = s->st;
  CK1(cudaMemsetAsync(s->J[0], 0, sizeof(float) * 3 * (s->nx + GC0 + GC1), st));
  s->j_cur = 0;
  for (auto &p : s->sp) {
    // window move of this species: decided on its counters after the push
    // (spec_move_window, particles.c:594-612)
    int shift = 0;
    if (s->mw) shift = ((float)(p.iter + 1) * s->dt) > (s->dx * (float)(p.n_move + 1)) ? 1 : 0;
    Push1 C;
    C.tem = (float)(0.5 * s->dt / p.m_q);
    C.dt_dx = s->dt / s->dx;
    C.qnx = p.q * s->dx / s->dt;
    C.q = p.q;
    C.nx = s->nx;
    C.shift = shift;
    C.open = (s->mw || s->part_open) ? 1 : 0;
    CK1(cudaMemsetAsync(p.d_ekin, 0, sizeof(double), st));
    const int pf = prof_begin(s, ZC1_K_PUSH);
    k1_push<<<grid_blocks(), 256, 0, st>>>(p.buf[p.cur], p.d_np, s->E, s->B, s->J[0], C, p.d_ekin, s->d_err);
    prof_end(s, pf);
    CK1(cudaGetLastError());
    s->launches += 1;
    if (C.open) TRY1(compact(s, p));
    p.iter += 1;
    if (shift) {
      p.n_move += 1;
      if (p.inj.type != 1) {
        TRY1(ensure_cap(s, p, p.inj.ppc));
        const int pi = prof_begin(s, ZC1_K_INJECT);
        k1_inject<<<1, 32, 0, st>>>(p.buf[p.cur], p.d_np, p.cap, p.inj, s->nx, p.n_move, s->d_err);
        prof_end(s, pi);
        CK1(cudaGetLastError());
        s->launches += 1;
        p.np_bound += p.inj.ppc;
      }
    }
    if (s->sort_every > 0 && p.iter % s->sort_every == 0) TRY1(sort_cells(s, p));
  }
  const int pc = prof_begin(s, ZC1_K_CURRENT);
  k1_current<<<1, 1024, 0, st>>>(s->J[0], s->J[1], s->nx, s->current_periodic, s->smooth, s->d_which);
  prof_end(s, pc);
  CK1(cudaGetLastError());
  s->launches += 1;
  s->j_cur = s->smooth.n % 2;  // the passes alternate buffers
  Emf1 M;
  M.nx = s->nx;
  M.dt = s->dt;
  M.dx = s->dx;
  M.bc = s->field_bc;
  s->iter += 1;
  M.shift = (s->mw && ((float)s->iter * s->dt) > (s->dx * (float)(s->n_move + 1))) ? 1 : 0;
  const int pe = prof_begin(s, ZC1_K_EMF);
  k1_emf<<<1, 1024, 0, st>>>(s->E, s->B, s->J[s->j_cur], s->mur, M);
  prof_end(s, pe);
  CK1(cudaGetLastError());
  s->launches += 1;
  if (M.shift) s->n_move += 1;
  return ZC_OK;
}

}  // namespace

extern "C" {

zc_status zc1_create(const zc1_desc *d, zc1_sim **out) {
  if (!d || !out) return fail1(ZC_EINVAL, "null argument");
  *out = nullptr;
  if (d->nx < 4) return fail1(ZC_EINVAL, "1-D grid needs at least 4 cells");
  if (!(d->box > 0) || !(d->dt > 0)) return fail1(ZC_EINVAL, "box and dt must be positive");
  const float dx = d->box / d->nx;
  if (d->dt >= dx) return fail1f(ZC_EINVAL, "Invalid timestep, courant condition violation, dtmax = %f", dx);
  zc1_sim *s = new (std::nothrow) zc1_sim;
  if (!s) return fail1(ZC_ENOMEM, "out of host memory");
  s->nx = d->nx;
  s->box = d->box;
  s->dx = dx;
  s->dt = d->dt;
  s->device = d->device;
  s->mw = d->moving_window ? 1 : 0;
  s->field_bc = s->mw ? 0 : (d->open_fields ? 2 : 1);
  s->current_periodic = s->mw ? 0 : 1;
  s->part_open = d->open_particles ? 1 : 0;
  s->sort_every = d->sort_every > 0 ? d->sort_every : 16;
  Guard1 g(s->device);
  const size_t gbytes = sizeof(float) * 3 * (s->nx + GC0 + GC1);
  cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&s->E, gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->B, gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->J[0], gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->J[1], gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->mur, sizeof(float) * 12);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_which, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_cnt, sizeof(int) * s->nx);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_emf, sizeof(double) * 6);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
  if (e == cudaSuccess) e = cudaMemset(s->E, 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->B, 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->J[0], 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->J[1], 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->mur, 0, sizeof(float) * 12);
  if (e == cudaSuccess) e = cudaMemset(s->d_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    zc1_destroy(s);
    return fail1f(ZC_ECUDA, "1-D simulation setup: %s", cudaGetErrorString(e));
  }
  *out = s;
  return ZC_OK;
}

void zc1_destroy(zc1_sim *s) {
  if (!s) return;
  Guard1 g(s->device);
  if (s->st) cudaStreamSynchronize(s->st);
  for (auto &p : s->sp) {
    free_parts(p.buf[0]);
    free_parts(p.buf[1]);
    cudaFree(p.d_np);
    cudaFree(p.d_ekin);
  }
  cudaFree(s->E);
  cudaFree(s->B);
  cudaFree(s->J[0]);
  cudaFree(s->J[1]);
  cudaFree(s->mur);
  cudaFree(s->d_which);
  cudaFree(s->d_err);
  cudaFree(s->d_blk);
  cudaFree(s->d_cnt);
  cudaFree(s->d_emf);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  for (cudaEvent_t e : s->prof_ev) cudaEventDestroy(e);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

zc_status zc1_add_species(zc1_sim *s, const zc1_species_desc *d, const zc1_part *parts, int np, int *id) {
  if (!s || !d || (np > 0 && !parts) || np < 0) return fail1(ZC_EINVAL, "invalid argument");
  if (s->mw && (d->uth[0] != 0 || d->uth[1] != 0 || d->uth[2] != 0))
    return fail1(ZC_EINVAL, "moving-window injection on the 1-D step supports cold species only");
  if (d->ppc <= 0) return fail1(ZC_EINVAL, "ppc must be positive");
  for (int i = 0; i < np; ++i)
    if (parts[i].ix < 0 || parts[i].ix >= s->nx) return fail1(ZC_EINVAL, "particle cell outside the grid");
  Guard1 g(s->device);
  Species1 p;
  p.m_q = d->m_q;
  p.q = d->q;
  p.inj.ppc = d->ppc;
  p.inj.type = d->density;
  p.inj.start = d->start;
  p.inj.end = d->end;
  p.inj.dx = s->dx;
  for (int c = 0; c < 3; ++c) p.inj.ufl[c] = d->ufl[c];
  p.cap = std::max(np + np / 4 + 1024, 1024);
  for (int b = 0; b < 2; ++b) TRY1(alloc_parts(p.buf[b], p.cap));
  CK1(cudaMalloc(&p.d_np, sizeof(int)));
  CK1(cudaMalloc(&p.d_ekin, sizeof(double)));
  CK1(cudaMemset(p.d_ekin, 0, sizeof(double)));
  // reference records (AoS) -> SoA
  std::vector<int> ix(np);
  std::vector<float> x(np), ux(np), uy(np), uz(np);
  for (int i = 0; i < np; ++i) {
    ix[i] = parts[i].ix;
    x[i] = parts[i].x;
    ux[i] = parts[i].ux;
    uy[i] = parts[i].uy;
    uz[i] = parts[i].uz;
  }
  if (np) {
    CK1(cudaMemcpy(p.buf[0].ix, ix.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
    CK1(cudaMemcpy(p.buf[0].x, x.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
    CK1(cudaMemcpy(p.buf[0].ux, ux.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
    CK1(cudaMemcpy(p.buf[0].uy, uy.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
    CK1(cudaMemcpy(p.buf[0].uz, uz.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
  }
  CK1(cudaMemcpy(p.d_np, &np, sizeof(int), cudaMemcpyHostToDevice));
  p.np_bound = np;
  s->sp.push_back(p);
  if (id) *id = (int)s->sp.size() - 1;
  return sort_cells(s, s->sp.back());
}

zc_status zc1_set_smooth(zc1_sim *s, int type, int level) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  if (type < 0 || type > 2) return fail1(ZC_EINVAL, "invalid smoothing type");
  if (type != 0 && level <= 0) return fail1(ZC_EINVAL, "Invalid smooth level along x direction");
  if (type != 0 && level > 15) return fail1(ZC_EINVAL, "smoothing level above 15 is not supported");
  Smooth1 S{};
  if (type != 0) {
    for (int i = 0; i < level; ++i) S.sa[S.n] = 0.25f, S.sb[S.n++] = 0.5f;
    if (type == 2) {
      // compensator [a, b, a] for n binomial passes (current.c:225-236)
      const float a = -1;
      const float b = (4.0 + 2.0 * level) / level;
      const float total = 2 * a + b;
      S.sa[S.n] = a / total, S.sb[S.n++] = b / total;
    }
  }
  s->smooth = S;
  return ZC_OK;
}

zc_status zc1_set_fields(zc1_sim *s, const float *E, const float *B) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  Guard1 g(s->device);
  const size_t gbytes = sizeof(float) * 3 * (s->nx + GC0 + GC1);
  if (E) CK1(cudaMemcpy(s->E, E, gbytes, cudaMemcpyHostToDevice));
  if (B) CK1(cudaMemcpy(s->B, B, gbytes, cudaMemcpyHostToDevice));
  return ZC_OK;
}

zc_status zc1_add_laser(zc1_sim *s, const zc_laser *in) {
  if (!s || !in) return fail1(ZC_EINVAL, "null argument");
  zc_laser L = *in;
  // parameter checks, em1d/emf.c:193-219
  if (L.fwhm != 0) {
    if (L.fwhm <= 0) return fail1(ZC_EINVAL, "Invalid laser FWHM, must be > 0");
    L.rise = L.fwhm;
    L.fall = L.fwhm;
    L.flat = 0.;
  }
  if (L.rise <= 0) return fail1(ZC_EINVAL, "Invalid laser RISE, must be > 0");
  if (L.flat < 0) return fail1(ZC_EINVAL, "Invalid laser FLAT, must be >= 0");
  if (L.fall <= 0) return fail1(ZC_EINVAL, "Invalid laser FALL, must be > 0");
  Guard1 g(s->device);
  zc::LaserConst c{};
  c.type = 0;
  c.start = L.start;
  c.rise = L.rise;
  c.flat = L.flat;
  c.fall = L.fall;
  c.a0 = L.a0;
  c.omega0 = L.omega0;
  c.polarization = L.polarization;
  c.dx = s->dx;
  k1_laser<<<1, 1024, 0, s->st>>>(s->E, s->B, s->nx, c, s->field_bc == 1 ? 1 : 0);
  CK1(cudaGetLastError());
  CK1(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc1_get_fields(zc1_sim *s, float *E, float *B) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  Guard1 g(s->device);
  const size_t gbytes = sizeof(float) * 3 * (s->nx + GC0 + GC1);
  CK1(cudaStreamSynchronize(s->st));
  if (E) CK1(cudaMemcpy(E, s->E, gbytes, cudaMemcpyDeviceToHost));
  if (B) CK1(cudaMemcpy(B, s->B, gbytes, cudaMemcpyDeviceToHost));
  return ZC_OK;
}

zc_status zc1_get_current(zc1_sim *s, float *J) {
  if (!s || !J) return fail1(ZC_EINVAL, "null argument");
  Guard1 g(s->device);
  CK1(cudaStreamSynchronize(s->st));
  CK1(cudaMemcpy(J, s->J[s->j_cur], sizeof(float) * 3 * (s->nx + GC0 + GC1), cudaMemcpyDeviceToHost));
  return ZC_OK;
}

zc_status zc1_step(zc1_sim *s, int nsteps) {
  if (!s || nsteps < 0) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  CK1(cudaEventRecord(s->ev0, s->st));
  for (int k = 0; k < nsteps; ++k) {
    TRY1(step1(s));
    if ((k + 1) % 16 == 0 && k + 1 < nsteps) {
      TRY1(check_err(s));
      prof_collect(s);
    }
  }
  CK1(cudaEventRecord(s->ev1, s->st));
  CK1(cudaEventSynchronize(s->ev1));
  cudaEventElapsedTime(&s->last_ms, s->ev0, s->ev1);
  prof_collect(s);
  return check_err(s);
}

zc_status zc1_set_profile(zc1_sim *s, int on) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  s->profile = on ? 1 : 0;
  for (int k = 0; k < ZC1_NKIND; ++k) {
    s->prof_ms[k] = 0.0;
    s->prof_n[k] = 0;
  }
  return ZC_OK;
}

zc_status zc1_get_profile(zc1_sim *s, double ms[ZC1_NKIND], long long launches[ZC1_NKIND]) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  for (int k = 0; k < ZC1_NKIND; ++k) {
    if (ms) ms[k] = s->prof_ms[k];
    if (launches) launches[k] = s->prof_n[k];
  }
  return ZC_OK;
}

zc_status zc1_get_launches(zc1_sim *s, long long *n) {
  if (!s || !n) return fail1(ZC_EINVAL, "null argument");
  *n = s->launches;
  return ZC_OK;
}

zc_status zc1_last_step_ms(zc1_sim *s, float *ms) {
  if (!s || !ms) return fail1(ZC_EINVAL, "null argument");
  *ms = s->last_ms;
  return ZC_OK;
}

zc_status zc1_energy(zc1_sim *s, double emf[6], double *kin) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  Guard1 g(s->device);
  if (emf) {
    k1_emf_energy<<<1, 1024, 0, s->st>>>(s->E, s->B, s->nx, s->dx, s->d_emf);
    CK1(cudaGetLastError());
    CK1(cudaMemcpyAsync(emf, s->d_emf, sizeof(double) * 6, cudaMemcpyDeviceToHost, s->st));
  }
  std::vector<double> k(s->sp.size());
  for (size_t i = 0; i < s->sp.size(); ++i)
    CK1(cudaMemcpyAsync(&k[i], s->sp[i].d_ekin, sizeof(double), cudaMemcpyDeviceToHost, s->st));
  CK1(cudaStreamSynchronize(s->st));
  if (kin)
    for (size_t i = 0; i < s->sp.size(); ++i) {
      // spec->energy = q m_q sum dx (particles.c:1034)
      const Species1 &p = s->sp[i];
      kin[i] = (double)(p.q * p.m_q) * k[i] * (double)s->dx;
    }
  return ZC_OK;
}

zc_status zc1_species_count(zc1_sim *s, int k, int *np) {
  if (!s || !np || k < 0 || k >= (int)s->sp.size()) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  *np = read_np(s, s->sp[k]);
  return ZC_OK;
}

zc_status zc1_get_particles(zc1_sim *s, int k, zc1_part *out, int cap, int *np) {
  if (!s || !np || k < 0 || k >= (int)s->sp.size()) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  Species1 &p = s->sp[k];
  const int n = read_np(s, p);
  *np = n;
  if (n > cap || (n > 0 && !out)) return fail1(ZC_EINVAL, "output buffer too small");
  std::vector<int> ix(n);
  std::vector<float> x(n), ux(n), uy(n), uz(n);
  if (n) {
    CK1(cudaMemcpy(ix.data(), p.buf[p.cur].ix, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(x.data(), p.buf[p.cur].x, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(ux.data(), p.buf[p.cur].ux, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(uy.data(), p.buf[p.cur].uy, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(uz.data(), p.buf[p.cur].uz, sizeof(float) * n, cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < n; ++i) out[i] = zc1_part{ix[i], x[i], ux[i], uy[i], uz[i]};
  return ZC_OK;
}

zc_status zc1_get_info(zc1_sim *s, int *iter, int *n_move) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  if (iter) *iter = s->iter;
  if (n_move) *n_move = s->n_move;
  return ZC_OK;
}

zc_status zc1_synchronize(zc1_sim *s) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  Guard1 g(s->device);
  CK1(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

}  // extern "C"
