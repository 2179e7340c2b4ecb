// zc_em1d.cu -- the em1d step on the GPU (libzpic_cuda, C-ABI zc1_*).
//
// Restates the reference's em1d time step (em1d/simulation.c:45-56):
// current_zero; per species the push -- gather (interpolate_fld,
// em1d/particles.c:864-894), relativistic Boris, move, 1-D zigzag deposit
// (dep_current_zamb, particles.c:707-790), window shift + cold injection and
// absorbing / periodic boundaries (particles.c:1040-1062, 594-612), cell
// sort every n_sort steps; then current_update (guard fold + binomial /
// compensated passes, em1d/current.c:111-330) and emf_advance (yee_b, yee_e,
// Mur, yee_b, guard cells, window shift, em1d/emf.c:379-580).
//
// Layout: particles are SoA arrays (ix, x, ux, uy, uz) in two buffers per
// species, kept in cell order by a counting sort every few steps so that the
// lanes of a warp share cells; E, B, J are the reference's float3 buffers
// (one lower and two upper guard cells).
//
// A step is two kernels.  The push runs one particle per lane: the current
// of a motion that stays in its cell is summed over the lanes of the cell
// (segmented warp reduction) and added to J with one float reduction per
// node (performed in L2); cell-crossing motions add their two segments
// directly.  With open boundaries or a moving window the survivors are
// appended to the other buffer (one atomic per warp), and the last CTA to
// finish injects the column the window uncovered and updates the species'
// device-resident state (buffer, counts, iteration, window moves, kinetic
// energy).  The fields kernel (one CTA; grids up to a few thousand cells
// in shared memory) folds and filters the current, advances E and B, moves
// the window and clears the deposit buffer for the next step.  Every
// decision of the step is taken on the device, so a block of n_sort steps
// ending with the cell sort is one CUDA graph, captured once and replayed.
//
// Compiled with --fmad=false: every float operation rounds as in the
// reference C, so particles advanced from the same fields land on the same
// bits.
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
// copies of the deposit buffer: the push's CTAs spread their float
// reductions over them (a 1-D grid is a few KB, held by few L2 slices), and
// the fields kernel sums them in a fixed order
constexpr int kJCopies = 8;
constexpr int kFieldUnroll = 2;  // grid elements per thread per load round of the fields kernel
enum { ERR1_ESCAPE = 1, ERR1_OVERFLOW = 2 };

struct Parts {
  int *ix;
  float *x, *ux, *uy, *uz;
};

// a species' state on the device, read and written only by the step's
// kernels (the host mirrors the counters, which it can predict)
struct SpecState1 {
  int np[2];        // particles in each buffer
  int cur;          // the buffer that holds the particles
  int iter;         // completed advances (spec->iter)
  int n_move;       // window moves (spec->n_move)
  unsigned done;    // CTAs finished in the running launch (0 between launches)
  double ekin_acc;  // kinetic-energy sum of the running advance
  double ekin;      // the sum of the last completed advance
  long long pushed;  // particles pushed so far (particle-steps)
};

struct Push1 {
  float tem, dt_dx, qnx, q;
  float dt, dx;  // window-move test (spec_move_window, particles.c:594-612)
  int nx;
  int mw;    // moving window
  int open;  // particles leaving [0, nx) are removed (open boundaries or window)
  int cap;   // capacity of each particle buffer
  int jstride;  // floats per deposit-buffer copy
};

// cold injection into column nx-1 after a window move (spec_set_x for
// uniform / step / slab profiles, particles.c:250-300; the momenta are ufl,
// the thermal part being zero)
struct Inject1 {
  int ppc, type;  // density type: 0 uniform, 1 empty, 2 step, 3 slab
  float start, end, dx;
  float ufl[3];
};

__device__ __forceinline__ float lerp1(const float *F, int i, int c, float w) {
  return F[(i + GC0) * 3 + c] * (1.0f - w) + F[(i + 1 + GC0) * 3 + c] * w;
}

// fire-and-forget float add performed in L2 (no value returned)
__device__ __forceinline__ void red(float *J, int i, int c, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(J + (i + GC0) * 3 + c), "f"(v) : "memory");
}

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

// adds a segment's contributions (an exact zero adds nothing and is skipped)
__device__ __forceinline__ void add_seg(float *J, int ix, const Seg1 &s) {
  if (s.jx != 0.f) red(J, ix, 0, s.jx);
  if (s.y0 != 0.f) red(J, ix, 1, s.y0);
  if (s.y1 != 0.f) red(J, ix + 1, 1, s.y1);
  if (s.z0 != 0.f) red(J, ix, 2, s.z0);
  if (s.z1 != 0.f) red(J, ix + 1, 2, s.z1);
}

// sums v over the lanes of each run of equal keys (lanes lane..run_last),
// leaving each run's sum in its first lane; maxlen: the longest run
__device__ __forceinline__ void run_sum(Seg1 &v, int run_last, unsigned maxlen) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    if ((unsigned)off >= maxlen) break;
    const bool take = lane + off <= run_last;
    const float o0 = __shfl_down_sync(0xffffffffu, v.jx, off);
    const float o1 = __shfl_down_sync(0xffffffffu, v.y0, off);
    const float o2 = __shfl_down_sync(0xffffffffu, v.y1, off);
    const float o3 = __shfl_down_sync(0xffffffffu, v.z0, off);
    const float o4 = __shfl_down_sync(0xffffffffu, v.z1, off);
    if (take) {
      v.jx += o0;
      v.y0 += o1;
      v.y1 += o2;
      v.z0 += o3;
      v.z1 += o4;
    }
  }
}


// ---------------------------------------------------------------------------
// push + deposit, one particle per lane, warps over consecutive particles;
// boundaries, compaction by append, and (last CTA) injection + bookkeeping
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k1_push(Parts b0, Parts b1, SpecState1 *st, const float *E, const float *B,
                                               float *Jall, Push1 C, Inject1 I, int *err) {
  __shared__ double sred[8];
  float *J = Jall + (size_t)(blockIdx.x % kJCopies) * C.jstride;
  __shared__ int s_last;
  const int cur = st->cur;
  const int n = st->np[cur];
  const int iter0 = st->iter, nmove0 = st->n_move;
  const int shift = (C.mw && ((float)(iter0 + 1) * C.dt) > (C.dx * (float)(nmove0 + 1))) ? 1 : 0;
  const Parts src = cur ? b1 : b0;
  const Parts dst = C.open ? (cur ? b0 : b1) : src;
  int *np_out = &st->np[1 - cur];
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
      ix = src.ix[i];
      x = src.x[i];
      ux = src.ux[i];
      uy = src.uy[i];
      uz = src.uz[i];
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
    // deposit (dep_current_zamb): qvy, qvz halved, split at the cell edge.
    // a: the motion inside cell ix (all of it, or its part up to the edge);
    // b: for a crossing, the part inside cell ix + di
    const float hy = qvy / 2.0f, hz = qvz / 2.0f;
    const bool split = valid && di != 0;
    Seg1 a, b = Seg1{0.f, 0.f, 0.f, 0.f, 0.f};
    if (split) {
      const int ib = (di == 1);
      const float delta = (x + dx - ib) / dx;
      b = seg_current(1 - ib, (x + dx) - di, dx * delta, hy * delta, hz * delta, C.qnx);
      a = seg_current(x, (float)ib, dx * (1.0f - delta), hy * (1.0f - delta), hz * (1.0f - delta), C.qnx);
    } else {
      a = seg_current(x, x + dx, dx, hy, hz, C.qnx);
    }
    // the lanes of a cell are contiguous (cell order): each part is summed
    // over the lanes of the cell and one lane per cell adds the sums, a to
    // cell ix, b to ix + 1 or ix - 1 (one sum per direction)
    {
      const int key = valid ? ix : -1 - lane;
      const int knext = __shfl_down_sync(0xffffffffu, key, 1);
      const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
      const unsigned lastmask = __ballot_sync(0xffffffffu, lane == 31 || knext != key);
      const int run_last = __ffs(lastmask & (0xffffffffu << lane)) - 1;
      const unsigned maxlen = __reduce_max_sync(0xffffffffu, (unsigned)(run_last - lane + 1));
      const bool head = valid && (lane == 0 || kprev != key);
      const unsigned up = __ballot_sync(0xffffffffu, split && di == 1);
      const unsigned down = __ballot_sync(0xffffffffu, split && di == -1);
      Seg1 sa = valid ? a : Seg1{0.f, 0.f, 0.f, 0.f, 0.f};
      run_sum(sa, run_last, maxlen);
      if (head) add_seg(J, ix, sa);
      if (up) {
        Seg1 sb = (di == 1) ? b : Seg1{0.f, 0.f, 0.f, 0.f, 0.f};
        run_sum(sb, run_last, maxlen);
        if (head) add_seg(J, ix + 1, sb);
      }
      if (down) {
        Seg1 sb = (di == -1) ? b : Seg1{0.f, 0.f, 0.f, 0.f, 0.f};
        run_sum(sb, run_last, maxlen);
        if (head) add_seg(J, ix - 1, sb);
      }
    }
    // boundaries (particles.c:1040-1062); with open boundaries the survivors
    // are appended to the other buffer, a warp at a time
    int nix = ix + di - shift;
    if (C.open) {
      const bool live = valid && nix >= 0 && nix < C.nx;
      const unsigned m = __ballot_sync(0xffffffffu, live);
      int obase = 0;
      if (lane == 0 && m) obase = atomicAdd(np_out, __popc(m));
      obase = __shfl_sync(0xffffffffu, obase, 0);
      if (live) {
        const int o = obase + __popc(m & ((1u << lane) - 1));
        if (o < C.cap) {
          dst.ix[o] = nix;
          dst.x[o] = x1;
          dst.ux[o] = ux;
          dst.uy[o] = uy;
          dst.uz[o] = uz;
        } else {
          errbits |= ERR1_OVERFLOW;
        }
      }
    } else if (valid) {
      nix += ((nix < 0) ? C.nx : 0) - ((nix >= C.nx) ? C.nx : 0);
      src.ix[i] = nix;
      src.x[i] = x1;
      src.ux[i] = ux;
      src.uy[i] = uy;
      src.uz[i] = uz;
    }
  }
  const double e = zc::block_sum_double<256>((double)ks - (double)kc, sred);
  if (threadIdx.x == 0 && e != 0.0) atomicAdd(&st->ekin_acc, e);
  if (errbits) atomicOr(err, errbits);
  // the last CTA to finish: every other CTA's stores and appends are done.
  // The barrier orders the CTA's writes before thread 0's fence, which is
  // cumulative, so one fence per CTA publishes them before the count.
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(&st->done, 1u) == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!s_last || threadIdx.x >= 32) return;
  __threadfence();
  int nn = C.open ? atomicAdd(np_out, 0) : n;
  if (shift && I.type != 1) {
    // spec_inject_particles into column nx-1 with the window's new offset
    const int ic = C.nx - 1;
    const float start = I.start / I.dx - (nmove0 + 1);
    const float end = I.end / I.dx - (nmove0 + 1);
    for (int k0 = 0; k0 < I.ppc; k0 += 32) {
      const int k = k0 + lane;
      const float pos = (float)((k + 0.5) / I.ppc);
      bool take = k < I.ppc;
      if (I.type == 2) take = take && ic + pos > start;
      if (I.type == 3) take = take && ic + pos > start && ic + pos < end;
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if (take) {
        const int o = nn + __popc(m & ((1u << lane) - 1));
        if (o < C.cap) {
          dst.ix[o] = ic;
          dst.x[o] = pos;
          dst.ux[o] = I.ufl[0];
          dst.uy[o] = I.ufl[1];
          dst.uz[o] = I.ufl[2];
        } else {
          atomicOr(err, ERR1_OVERFLOW);
        }
      }
      nn += __popc(m);
    }
  }
  if (lane == 0) {
    if (nn > C.cap) {
      nn = C.cap;
      atomicOr(err, ERR1_OVERFLOW);
    }
    if (C.open) {
      st->np[1 - cur] = nn;
      st->np[cur] = 0;
      st->cur = 1 - cur;
    } else if (nn != n) {
      st->np[cur] = nn;
    }
    st->ekin = *(volatile double *)&st->ekin_acc;
    st->ekin_acc = 0.0;
    st->iter = iter0 + 1;
    st->n_move = nmove0 + shift;
    st->pushed += n;
    __threadfence();
    st->done = 0u;
  }
}

// ---------------------------------------------------------------------------
// counting sort by cell (spec_sort, particles.c:796-843) from the current
// buffer into the other: counts and cursors over nx cells, warp-aggregated
// atomics (the input is mostly sorted already); the scatter's last CTA
// switches the buffers
// ---------------------------------------------------------------------------
__global__ void k1_cell_count(Parts b0, Parts b1, const SpecState1 *st, int *cnt) {
  const int cur = st->cur;
  const int n = st->np[cur];
  const int *ix = cur ? b1.ix : b0.ix;
  for (int b = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b < n; b += gridDim.x * blockDim.x) {
    const int i = b + (threadIdx.x & 31);
    const int key = i < n ? ix[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (i < n && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[key], __popc(peers));
  }
}

__global__ void k1_cell_scan(int *cnt, int nx, SpecState1 *st) {
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
  if (threadIdx.x == 0) st->np[1 - st->cur] = st->np[st->cur];
}

__global__ void k1_cell_scatter(Parts b0, Parts b1, SpecState1 *st, int *cursor) {
  __shared__ int s_last;
  const int cur = st->cur;
  const int n = st->np[cur];
  const Parts src = cur ? b1 : b0, dst = cur ? b0 : b1;
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
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(&st->done, 1u) == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    st->np[cur] = 0;
    st->cur = 1 - cur;
    __threadfence();
    st->done = 0u;
  }
}

// ---------------------------------------------------------------------------
// current update + field advance, one CTA (current.c:111-330, emf.c:379-580)
// ---------------------------------------------------------------------------
struct Smooth1 {
  int n;
  float sa[16], sb[16];
};

struct Fields1 {
  int nx;
  float dt, dx;
  int bc;            // 0 none, 1 periodic, 2 open (Mur)
  int cur_periodic;  // periodic guard fold of the current
  int mw;            // moving window
  Smooth1 S;
};

// the field's own counters on the device (emf->iter, emf->n_move)
struct FieldState1 {
  int iter, n_move;
};

__device__ __forceinline__ void yee_b1(const float *E, float *B, int nx, float dt_dx) {
  for (int i = (int)threadIdx.x - 1; i <= nx; i += blockDim.x) {
    const int k = (i + GC0) * 3;
    B[k + 1] += (dt_dx * (E[k + 3 + 2] - E[k + 2]));
    B[k + 2] += (-dt_dx * (E[k + 3 + 1] - E[k + 1]));
  }
}

__device__ __forceinline__ void yee_e1(float *E, const float *B, const float *J, int nx, float dt, float dt_dx) {
  for (int i = threadIdx.x; i <= nx + 1; i += blockDim.x) {
    const int k = (i + GC0) * 3;
    E[k + 0] += (-dt * J[k + 0]);
    E[k + 1] += (-dt_dx * (B[k + 2] - B[k - 3 + 2]) - dt * J[k + 1]);
    E[k + 2] += (+dt_dx * (B[k + 1] - B[k - 3 + 1]) - dt * J[k + 2]);
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

// SM: the four grids (two current buffers, E, B) live in shared memory for
// the whole kernel, else the kernel works on the global buffers (Jdep and
// Jout then serve as the filter's two buffers).  Jdep (kJCopies copies,
// summed first) is left zero for the next step's deposit; Jout holds the
// filtered current.
template <bool SM>
__global__ void __launch_bounds__(1024) k1_fields(float *E, float *B, float *Jdep, float *Jout, float *mur,
                                                  FieldState1 *fs, Fields1 M) {
  extern __shared__ float smem[];
  const int nx = M.nx;
  const int nf = (nx + GC0 + GC1) * 3;
  const int iter = fs->iter + 1, nmove0 = fs->n_move;
  float *ja, *jb, *e, *b;
  if (SM) {
    ja = smem;
    jb = smem + nf;
    e = smem + 2 * nf;
    b = smem + 3 * nf;
    // every load of a round is issued before its stores (one L2 round trip
    // per kFieldUnroll x blockDim.x elements)
    for (int k0 = threadIdx.x; k0 < nf; k0 += kFieldUnroll * blockDim.x) {
      float v[kFieldUnroll][kJCopies], ve[kFieldUnroll], vb[kFieldUnroll];
#pragma unroll
      for (int r = 0; r < kFieldUnroll; ++r) {
        const int k = k0 + r * blockDim.x;
        const bool in = k < nf;
#pragma unroll
        for (int c = 0; c < kJCopies; ++c) v[r][c] = in ? Jdep[c * nf + k] : 0.f;
        ve[r] = in ? E[k] : 0.f;
        vb[r] = in ? B[k] : 0.f;
      }
#pragma unroll
      for (int r = 0; r < kFieldUnroll; ++r) {
        const int k = k0 + r * blockDim.x;
        if (k < nf) {
          float sum = 0.f;
#pragma unroll
          for (int c = 0; c < kJCopies; ++c) {
            sum += v[r][c];
            Jdep[c * nf + k] = 0.f;
          }
          ja[k] = sum;
          e[k] = ve[r];
          b[k] = vb[r];
        }
      }
    }
  } else {
    ja = Jdep;
    jb = Jout;
    e = E;
    b = B;
    for (int k = threadIdx.x; k < nf; k += blockDim.x) {
      float v = 0.f;
#pragma unroll
      for (int c = 0; c < kJCopies; ++c) {
        v += Jdep[c * nf + k];
        if (c) Jdep[c * nf + k] = 0.f;
      }
      Jdep[k] = v;
    }
  }
  __syncthreads();
  // current_update_gc: J[i] += J[nx + i] for i = -1, 0, 1, then the upper
  // cells copy the lower (current.c:112-132)
  float *J = ja, *O = jb;
  if (M.cur_periodic) {
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
  // the filter passes [sa, sb, sa] (kernel_x, current.c:265-297), out of place
  for (int p = 0; p < M.S.n; ++p) {
    const float sa = M.S.sa[p], sb = M.S.sb[p];
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
      O[(gi + GC0) * 3 + c] = M.cur_periodic ? O[(src + GC0) * 3 + c] : J[(gi + GC0) * 3 + c];
    }
    __syncthreads();
    float *t = J;
    J = O;
    O = t;
  }
  // the filtered current for reports
  if (SM) {
    for (int k = threadIdx.x; k < nf; k += blockDim.x) Jout[k] = J[k];
  } else if (J != Jout) {
    for (int k = threadIdx.x; k < nf; k += blockDim.x) Jout[k] = J[k];
    __syncthreads();
    J = Jout;
  }
  // emf_advance (emf.c:548-566)
  const float hdt = M.dt / 2.0f;
  yee_b1(e, b, nx, hdt / M.dx);
  __syncthreads();
  yee_e1(e, b, J, nx, M.dt, M.dt / M.dx);
  __syncthreads();
  if (M.bc == 2 && threadIdx.x == 0) {
    // first-order Mur (mur_abc, emf.c:379-415); mur = fld[2][3], tmp[2][3]
    float *fld = mur, *tmp = mur + 6;
    const float S = (M.dt - M.dx) / (M.dt + M.dx);
    const int lo = (0 + GC0) * 3, hi = (nx - 1 + GC0) * 3;
    fld[1] = tmp[1] + S * (e[lo + 1] - fld[1]);
    fld[2] = tmp[2] + S * (e[lo + 2] - fld[2]);
    e[(-1 + GC0) * 3 + 1] = fld[1];
    e[(-1 + GC0) * 3 + 2] = fld[2];
    tmp[1] = e[lo + 1];
    tmp[2] = e[lo + 2];
    fld[4] = tmp[4] + S * (e[hi + 1] - fld[4]);
    fld[5] = tmp[5] + S * (e[hi + 2] - fld[5]);
    e[(nx + GC0) * 3 + 1] = fld[4];
    e[(nx + GC0) * 3 + 2] = fld[5];
    tmp[4] = e[hi + 1];
    tmp[5] = e[hi + 2];
  }
  __syncthreads();
  yee_b1(e, b, nx, hdt / M.dx);
  __syncthreads();
  if (M.bc == 1) periodic_gc1(e, b, nx);
  if (!SM)
    for (int k = threadIdx.x; k < nf; k += blockDim.x) Jdep[k] = 0.f;
  __syncthreads();
  // window shift (emf_move_window, emf.c:513-540): cells move left by one,
  // cells nx-1 .. nx+1 become zero
  const int shift = (M.mw && ((float)iter * M.dt) > (M.dx * (float)(nmove0 + 1))) ? 1 : 0;
  if (SM) {
    for (int k = threadIdx.x; k < nf; k += blockDim.x) {
      E[k] = shift ? ((k < nx * 3) ? e[k + 3] : 0.f) : e[k];
      B[k] = shift ? ((k < nx * 3) ? b[k + 3] : 0.f) : b[k];
    }
  } else if (shift) {
    for (int base = 0; base < nf; base += blockDim.x) {
      // E[k] <- E[k + 3] for k < nf - 3, every value read before any write
      const int k = base + threadIdx.x;
      float ve = 0.f, vb = 0.f;
      if (k < nf - 3) {
        ve = E[k + 3];
        vb = B[k + 3];
      }
      __syncthreads();
      if (k < nf - 3) {
        E[k] = ve;
        B[k] = vb;
      }
      __syncthreads();
    }
    for (int k = nx * 3 + threadIdx.x; k < nf; k += blockDim.x) {
      E[k] = 0.f;
      B[k] = 0.f;
    }
  }
  if (threadIdx.x == 0) {
    fs->iter = iter;
    fs->n_move = nmove0 + shift;
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
  int iter = 0, n_move = 0;  // mirrors of the device counters
  int cap = 0;
  long long np_bound = 0;    // upper bound of the device count
  Parts buf[2] = {};
  SpecState1 *d_st = nullptr;
};

}  // namespace zc1

using namespace zc1;

struct zc1_sim {
  int nx;
  float box, dx, dt;
  int device;
  int field_bc, current_periodic, part_open, mw, sort_every;
  int push_ctas = 0;         // cap of the push's CTAs (0: one wave)
  int iter = 0, n_move = 0;  // mirrors of the field's device counters
  Smooth1 smooth{};
  cudaStream_t st = nullptr;
  float *E = nullptr, *B = nullptr, *Jdep = nullptr, *Jout = nullptr, *mur = nullptr;
  FieldState1 *d_fs = nullptr;
  int *d_err = nullptr, *d_cnt = nullptr;
  double *d_emf = nullptr;
  size_t fields_smem = 0;  // dynamic shared memory of the fields kernel (0: global variant)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  int timing = 0;          // steps enqueued since ev0, not yet waited for
  long long launches = 0;  // kernels launched by the steps so far
  // the captured block of sort_every steps (the last one sorts), and the
  // same block with an event pair around every kernel for profiling
  cudaGraphExec_t block = nullptr, block_prof = nullptr;
  int block_kernels = 0, block_prof_kernels = 0;
  size_t prof_graph_slots = 0;  // event pairs the profiling graph records
  int capturing = 0;
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

constexpr int kPushThreads = 256;
constexpr int kMaxCtas = 152 * 4;  // the push CTAs resident together (4 per SM)

// CTAs of the push: one particle per thread, up to one wave, or up to the
// simulation's own cap (simulations that share the GPU leave each other room)
int push_blocks(const zc1_sim *s, int cap) {
  const int most = s->push_ctas > 0 ? std::min(s->push_ctas, kMaxCtas) : kMaxCtas;
  return std::max(1, std::min(most, (cap + kPushThreads - 1) / kPushThreads));
}

int sort_blocks(const zc1_sim *s) { return s->push_ctas > 0 ? std::min(s->push_ctas, kMaxCtas) : kMaxCtas; }

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

zc_status read_state(zc1_sim *s, const Species1 &p, SpecState1 &h) {
  CK1(cudaMemcpyAsync(&h, p.d_st, sizeof(SpecState1), cudaMemcpyDeviceToHost, s->st));
  CK1(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

void drop_graph(zc1_sim *s) {
  if (s->block) cudaGraphExecDestroy(s->block);
  if (s->block_prof) cudaGraphExecDestroy(s->block_prof);
  s->block = s->block_prof = nullptr;
  s->block_kernels = s->block_prof_kernels = 0;
  s->prof_graph_slots = 0;
  s->prof_used = 0;
}

zc_status check_err(zc1_sim *s) {
  int e = 0;
  CK1(cudaMemcpyAsync(&e, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK1(cudaStreamSynchronize(s->st));
  if (e & ERR1_OVERFLOW) return fail1(ZC_EOVERFLOW, "1-D particle buffer full at injection");
  if (e & ERR1_ESCAPE) return fail1(ZC_EPARTICLE_ESCAPE, "a particle moved a cell or more, or left the grid");
  return ZC_OK;
}

// room for `steps` more steps of injection in both buffers of every species, keeping
// the current ones; the device count is read (a sync) only when its upper
// bound no longer fits, and the buffers grow only when the true count does
// not (which also drops the captured graph: it holds the old buffers)
zc_status ensure_cap(zc1_sim *s, int steps) {
  for (auto &p : s->sp) {
    // at most one window move, hence one injected column, per step
    const long long extra = (s->mw && p.inj.type != 1) ? (long long)steps * p.inj.ppc : 0;
    if (p.np_bound + extra <= p.cap) continue;
    SpecState1 h;
    TRY1(read_state(s, p, h));
    TRY1(check_err(s));
    const int n = h.np[h.cur];
    p.np_bound = n;
    if (n + extra <= p.cap) continue;
    const long long want = std::max<long long>(n + extra, (long long)(1.25 * n) + 1024 + extra);
    if (want > (1LL << 30)) return fail1(ZC_EOVERFLOW, "1-D particle buffer above 2^30 particles");
    const int cap = (int)want;
    Parts nb[2];
    for (int b = 0; b < 2; ++b) TRY1(alloc_parts(nb[b], cap));
    TRY1(copy_parts(p.buf[h.cur], nb[0], n, s->st));
    h.np[0] = n;
    h.np[1] = 0;
    h.cur = 0;
    CK1(cudaMemcpyAsync(p.d_st, &h, sizeof(SpecState1), cudaMemcpyHostToDevice, s->st));
    CK1(cudaStreamSynchronize(s->st));
    free_parts(p.buf[0]);
    free_parts(p.buf[1]);
    p.buf[0] = nb[0];
    p.buf[1] = nb[1];
    p.cap = cap;
    drop_graph(s);
  }
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
  // inside a capture the record becomes a graph node that records the event
  // each time the graph runs
  if (s->capturing)
    cudaEventRecordWithFlags(s->prof_ev[2 * slot], s->st, cudaEventRecordExternal);
  else
    cudaEventRecord(s->prof_ev[2 * slot], s->st);
  s->prof_used = slot + 1;
  return (int)slot;
}

void prof_end(zc1_sim *s, int slot) {
  if (slot < 0) return;
  if (s->capturing)
    cudaEventRecordWithFlags(s->prof_ev[2 * (size_t)slot + 1], s->st, cudaEventRecordExternal);
  else
    cudaEventRecord(s->prof_ev[2 * (size_t)slot + 1], s->st);
}

// adds the launches recorded in slots [from, to) to the per-kind sums (after
// a stream sync)
void prof_add(zc1_sim *s, size_t from, size_t to) {
  for (size_t i = from; i < to; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s->prof_ev[2 * i], s->prof_ev[2 * i + 1]) == cudaSuccess) {
      s->prof_ms[s->prof_kind[i]] += ms;
      s->prof_n[s->prof_kind[i]] += 1;
    }
  }
}

// the eager launches recorded since the last collection (the profiling
// graph keeps the first prof_graph_slots slots)
void prof_collect(zc1_sim *s) {
  if (s->prof_used > s->prof_graph_slots) prof_add(s, s->prof_graph_slots, s->prof_used);
  s->prof_used = s->prof_graph_slots;
}

// enqueues the cell sort of species p (3 kernels); returns the kernel count
int enqueue_sort(zc1_sim *s, Species1 &p) {
  const int pf = prof_begin(s, ZC1_K_SORT);
  cudaMemsetAsync(s->d_cnt, 0, sizeof(int) * s->nx, s->st);
  k1_cell_count<<<sort_blocks(s), 256, 0, s->st>>>(p.buf[0], p.buf[1], p.d_st, s->d_cnt);
  k1_cell_scan<<<1, 1024, 0, s->st>>>(s->d_cnt, s->nx, p.d_st);
  k1_cell_scatter<<<sort_blocks(s), 256, 0, s->st>>>(p.buf[0], p.buf[1], p.d_st, s->d_cnt);
  prof_end(s, pf);
  return 3;
}

// enqueues one step (sim_iter): the push of every species (each followed by
// its cell sort when `sort`), then the fields kernel; nothing is decided on
// the host, so the same calls serve eager steps and graph capture.  Returns
// the kernel count.
int enqueue_step(zc1_sim *s, bool sort) {
  int k = 0;
  for (auto &p : s->sp) {
    Push1 C;
    C.tem = (float)(0.5 * s->dt / p.m_q);
    C.dt_dx = s->dt / s->dx;
    C.qnx = p.q * s->dx / s->dt;
    C.q = p.q;
    C.dt = s->dt;
    C.dx = s->dx;
    C.nx = s->nx;
    C.mw = s->mw;
    C.open = (s->mw || s->part_open) ? 1 : 0;
    C.cap = p.cap;
    C.jstride = 3 * (s->nx + GC0 + GC1);
    const int pf = prof_begin(s, ZC1_K_PUSH);
    k1_push<<<push_blocks(s, p.cap), kPushThreads, 0, s->st>>>(p.buf[0], p.buf[1], p.d_st, s->E, s->B, s->Jdep, C,
                                                            p.inj, s->d_err);
    prof_end(s, pf);
    k += 1;
    if (sort) k += enqueue_sort(s, p);
  }
  Fields1 M;
  M.nx = s->nx;
  M.dt = s->dt;
  M.dx = s->dx;
  M.bc = s->field_bc;
  M.cur_periodic = s->current_periodic;
  M.mw = s->mw;
  M.S = s->smooth;
  const int pf = prof_begin(s, ZC1_K_FIELDS);
  if (s->fields_smem)
    k1_fields<true><<<1, 1024, s->fields_smem, s->st>>>(s->E, s->B, s->Jdep, s->Jout, s->mur, s->d_fs, M);
  else
    k1_fields<false><<<1, 1024, 0, s->st>>>(s->E, s->B, s->Jdep, s->Jout, s->mur, s->d_fs, M);
  prof_end(s, pf);
  return k + 1;
}

// the host's mirror of one step's counters (the device takes the same
// decisions from the same float arithmetic)
void advance_mirror(zc1_sim *s) {
  for (auto &p : s->sp) {
    const int shift = (s->mw && ((float)(p.iter + 1) * s->dt) > (s->dx * (float)(p.n_move + 1))) ? 1 : 0;
    p.iter += 1;
    p.n_move += shift;
    if (shift && p.inj.type != 1) p.np_bound += p.inj.ppc;
  }
  s->iter += 1;
  if (s->mw && ((float)s->iter * s->dt) > (s->dx * (float)(s->n_move + 1))) s->n_move += 1;
}

// sort after this step's push: spec->iter (after the advance) a multiple of n_sort
bool sorts_next(const zc1_sim *s, const Species1 &p) {
  return s->sort_every > 0 && (p.iter + 1) % s->sort_every == 0;
}

// one step launched directly (species share their iteration count: they are
// added before the first advance)
zc_status step_eager(zc1_sim *s) {
  TRY1(ensure_cap(s, 1));
  s->launches += enqueue_step(s, !s->sp.empty() && sorts_next(s, s->sp[0]));
  CK1(cudaGetLastError());
  advance_mirror(s);
  return ZC_OK;
}

// a block of sort_every steps ending with the sort, as one graph
zc_status run_block(zc1_sim *s) {
  const int nb = s->sort_every;
  TRY1(ensure_cap(s, nb));
  cudaGraphExec_t &exec = s->profile ? s->block_prof : s->block;
  int &kernels = s->profile ? s->block_prof_kernels : s->block_kernels;
  if (!exec) {
    if (s->profile) {
      CK1(cudaStreamSynchronize(s->st));
      prof_collect(s);
      s->prof_graph_slots = 0;
      s->prof_used = 0;
    }
    cudaGraph_t g = nullptr;
    CK1(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    s->capturing = 1;
    int k = 0;
    for (int i = 0; i < nb; ++i) k += enqueue_step(s, i == nb - 1);
    s->capturing = 0;
    const cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (e != cudaSuccess) return fail1f(ZC_ECUDA, "1-D step capture: %s", cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      exec = nullptr;
      return fail1f(ZC_ECUDA, "1-D step graph: %s", cudaGetErrorString(ei));
    }
    kernels = k;
    if (s->profile) s->prof_graph_slots = s->prof_used;
  }
  CK1(cudaGraphLaunch(exec, s->st));
  s->launches += kernels;
  if (s->profile) {
    // the graph records the same events at every replay: read them now
    CK1(cudaStreamSynchronize(s->st));
    prof_add(s, 0, s->prof_graph_slots);
  }
  for (int i = 0; i < nb; ++i) advance_mirror(s);
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
  s->push_ctas = d->push_ctas > 0 ? d->push_ctas : 0;
  Guard1 g(s->device);
  const size_t gbytes = sizeof(float) * 3 * (s->nx + GC0 + GC1);
  cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&s->E, gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->B, gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->Jdep, gbytes * kJCopies);
  if (e == cudaSuccess) e = cudaMalloc(&s->Jout, gbytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->mur, sizeof(float) * 12);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_fs, sizeof(FieldState1));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_cnt, sizeof(int) * s->nx);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_emf, sizeof(double) * 6);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
  if (e == cudaSuccess) e = cudaMemset(s->E, 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->B, 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->Jdep, 0, gbytes * kJCopies);
  if (e == cudaSuccess) e = cudaMemset(s->Jout, 0, gbytes);
  if (e == cudaSuccess) e = cudaMemset(s->mur, 0, sizeof(float) * 12);
  if (e == cudaSuccess) e = cudaMemset(s->d_fs, 0, sizeof(FieldState1));
  if (e == cudaSuccess) e = cudaMemset(s->d_err, 0, sizeof(int));
  // the fields kernel keeps its four grids in shared memory when they fit.
  // Its dynamic shared-memory ceiling is a property of the kernel for the
  // whole process, so it is raised to the device's maximum (a ceiling, not an
  // allocation) rather than to this grid's size, which could lower it below
  // what another simulation launches with.
  int optin = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device);
  const size_t smem = 4 * gbytes;
  if (e == cudaSuccess && smem <= (size_t)optin) {
    e = cudaFuncSetAttribute(k1_fields<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) s->fields_smem = smem;
  }
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
  drop_graph(s);
  for (auto &p : s->sp) {
    free_parts(p.buf[0]);
    free_parts(p.buf[1]);
    cudaFree(p.d_st);
  }
  cudaFree(s->E);
  cudaFree(s->B);
  cudaFree(s->Jdep);
  cudaFree(s->Jout);
  cudaFree(s->mur);
  cudaFree(s->d_fs);
  cudaFree(s->d_err);
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
  if (!s->sp.empty() && s->sp[0].iter != 0)
    return fail1(ZC_EINVAL, "species are added to the 1-D step before its first advance");
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
  // a window that injects fills up to about nx * ppc particles: room for
  // that from the start keeps the host from reading the count back (a wait
  // on the stream) while the window fills
  long long want = std::max(np + np / 4 + 1024, 1024);
  if (s->mw && d->density != 1) want = std::max(want, (long long)(1.25 * s->nx * d->ppc) + 1024);
  if (want > (1LL << 30)) return fail1(ZC_EOVERFLOW, "1-D particle buffer above 2^30 particles");
  p.cap = (int)want;
  for (int b = 0; b < 2; ++b) TRY1(alloc_parts(p.buf[b], p.cap));
  CK1(cudaMalloc(&p.d_st, sizeof(SpecState1)));
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
  SpecState1 h{};
  h.np[0] = np;
  CK1(cudaMemcpy(p.d_st, &h, sizeof(SpecState1), cudaMemcpyHostToDevice));
  p.np_bound = np;
  s->sp.push_back(p);
  drop_graph(s);
  if (id) *id = (int)s->sp.size() - 1;
  // cell order for the warp reduction of the first steps
  s->launches += enqueue_sort(s, s->sp.back());
  CK1(cudaGetLastError());
  CK1(cudaStreamSynchronize(s->st));
  return ZC_OK;
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
      // compensator [a, b, a] for n binomial passes (get_smooth_comp, current.c:244-253)
      const float a = -1;
      const float b = (4.0 + 2.0 * level) / level;
      const float total = 2 * a + b;
      S.sa[S.n] = a / total, S.sb[S.n++] = b / total;
    }
  }
  s->smooth = S;
  drop_graph(s);
  return ZC_OK;
}

zc_status zc1_set_fields(zc1_sim *s, const float *E, const float *B) {
  if (!s) return fail1(ZC_EINVAL, "null simulation handle");
  Guard1 g(s->device);
  const size_t gbytes = sizeof(float) * 3 * (s->nx + GC0 + GC1);
  CK1(cudaStreamSynchronize(s->st));
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
  CK1(cudaMemcpy(J, s->Jout, sizeof(float) * 3 * (s->nx + GC0 + GC1), cudaMemcpyDeviceToHost));
  return ZC_OK;
}

zc_status zc1_step_async(zc1_sim *s, int nsteps) {
  if (!s || nsteps < 0) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  if (!s->timing) {
    CK1(cudaEventRecord(s->ev0, s->st));
    s->timing = 1;
  }
  int k = 0;
  while (k < nsteps) {
    const bool aligned = !s->sp.empty() && s->sort_every > 0 && s->sp[0].iter % s->sort_every == 0;
    if (aligned && nsteps - k >= s->sort_every) {
      TRY1(run_block(s));
      k += s->sort_every;
    } else {
      TRY1(step_eager(s));
      k += 1;
    }
    if (s->profile && s->prof_used >= s->prof_graph_slots + 4096) {
      CK1(cudaStreamSynchronize(s->st));
      prof_collect(s);
    }
  }
  return ZC_OK;
}

zc_status zc1_step(zc1_sim *s, int nsteps) {
  TRY1(zc1_step_async(s, nsteps));
  return zc1_synchronize(s);
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
  std::vector<SpecState1> h(s->sp.size());
  for (size_t i = 0; i < s->sp.size(); ++i)
    CK1(cudaMemcpyAsync(&h[i], s->sp[i].d_st, sizeof(SpecState1), cudaMemcpyDeviceToHost, s->st));
  CK1(cudaStreamSynchronize(s->st));
  if (kin)
    for (size_t i = 0; i < s->sp.size(); ++i) {
      // spec->energy = q m_q sum dx (particles.c:1038)
      const Species1 &p = s->sp[i];
      kin[i] = (double)(p.q * p.m_q) * h[i].ekin * (double)s->dx;
    }
  return ZC_OK;
}

zc_status zc1_species_count(zc1_sim *s, int k, int *np) {
  if (!s || !np || k < 0 || k >= (int)s->sp.size()) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  SpecState1 h;
  TRY1(read_state(s, s->sp[k], h));
  *np = h.np[h.cur];
  s->sp[k].np_bound = *np;
  return ZC_OK;
}

zc_status zc1_get_particles(zc1_sim *s, int k, zc1_part *out, int cap, int *np) {
  if (!s || !np || k < 0 || k >= (int)s->sp.size()) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  Species1 &p = s->sp[k];
  SpecState1 h;
  TRY1(read_state(s, p, h));
  const int n = h.np[h.cur];
  const Parts &b = p.buf[h.cur];
  *np = n;
  if (n > cap || (n > 0 && !out)) return fail1(ZC_EINVAL, "output buffer too small");
  std::vector<int> ix(n);
  std::vector<float> x(n), ux(n), uy(n), uz(n);
  if (n) {
    CK1(cudaMemcpy(ix.data(), b.ix, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(x.data(), b.x, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(ux.data(), b.ux, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(uy.data(), b.uy, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CK1(cudaMemcpy(uz.data(), b.uz, sizeof(float) * n, cudaMemcpyDeviceToHost));
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
  if (s->timing) {
    CK1(cudaEventRecord(s->ev1, s->st));
    CK1(cudaEventSynchronize(s->ev1));
    cudaEventElapsedTime(&s->last_ms, s->ev0, s->ev1);
    s->timing = 0;
  }
  CK1(cudaStreamSynchronize(s->st));
  prof_collect(s);
  return check_err(s);
}

zc_status zc1_species_pushed(zc1_sim *s, int k, long long *pushed) {
  if (!s || !pushed || k < 0 || k >= (int)s->sp.size()) return fail1(ZC_EINVAL, "invalid argument");
  Guard1 g(s->device);
  SpecState1 h;
  TRY1(read_state(s, s->sp[k], h));
  *pushed = h.pushed;
  return ZC_OK;
}

}  // extern "C"
