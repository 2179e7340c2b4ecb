// zc_kernels.h -- launch interface between the host runtime (zc_api.cu) and
// the kernels (zc_particles.cu, zc_fields.cu).
#pragma once

#include <algorithm>

#include "zc_internal.cuh"

namespace zc {

struct PushConst {
  float tem, dt_dx, dt_dy, qnx, qny, q;   // particles.c:1111-1117
  int nx, ny, ntx, nty;
  int shift;                              // moving-window shift applied this step (0/1)
  int mw;                                 // absorbing boundaries along x
  // tile current as integers (see jsplit): a contribution v counts as
  // rint(v js) = h 2^2L + m 2^L + l; js_invl = 2^-L, js_twol = 2^L,
  // js_inv2l = 2^-2L, js_two2l = 2^2L, js_lo = 1 / js; deterministic global
  // sums in units of 2^-40 take each integer times js_det (2^40 / js)
  float js, js_invl, js_twol, js_inv2l, js_two2l, js_lo;
  int js_l;
  long long js_det;
};

struct TileSet {
  const int *off, *cap;
  int *np;
  int ntiles;
};

struct Outbox {                           // particles leaving a tile, per tile `cap` slots
  Particles p;
  int *dst, *cnt;
  int cap;
};

struct Spill {                            // particles without room in a tile
  Particles p;
  int *cnt;
  int cap;
};

struct LayoutConst {
  int TX, TY, ntx, nty, nx, ny;
};

// Deterministic mode: the current is accumulated as 64-bit fixed point,
// every contribution rounded once to a multiple of 2^-40.  Integer sums are
// exact, so the result does not depend on the order of the additions (warp
// order, atomics, tiles, spill list): runs are bit-reproducible.  Range:
// |J| < 2^23 per cell and component.  Kinetic-energy terms are split into a
// multiple of 2^-30 and a remainder counted in units of 2^-62, each summed
// as a 64-bit integer (range 2^33, resolution 2^-62).
struct FixedJ {
  unsigned long long *p;  // 3 planes laid out as the float J planes
  int pitch;
  size_t plane;
  float *f;               // the float J planes (the push's direct deposits)
};
constexpr double kJFixScale = 1099511627776.0;         // 2^40
constexpr double kEFixHi = 1073741824.0;                 // 2^30
constexpr double kEFixLo = 4611686018427387904.0;        // 2^62

// a float kinetic-energy term as two integers: hi = rint(v 2^30) and lo =
// rint((v - hi 2^-30) 2^62), without double arithmetic: t = v 2^30 is exact,
// so are its nearest integer hf and the remainder t - hf (|.| <= 1/2), and
// the remainder times 2^32 is lo (exact for v >= 2^-39, rounded below)
__device__ __forceinline__ void efix_split(float v, long long &hi, long long &lo) {
  const float t = __fmul_rn(v, 1073741824.0f);  // 2^30
  const float hf = rintf(t);
  hi = __float2ll_rn(hf);
  lo = __float2ll_rn(__fmul_rn(__fsub_rn(t, hf), 4294967296.0f));  // 2^32
}
__host__ __device__ __forceinline__ double efix_join(long long hi, long long lo) {
  return (double)hi / kEFixHi + (double)lo / kEFixLo;
}

struct PushLaunch {
  const CUtensorMap *tm_eb;
  Particles pin, pout;
  TileSet T;
  Outbox Oin, O;                          // pending incoming (previous step), leavers (this step)
  Spill S;
  double *ekin_tile;
  int *err;
  PushConst C;
  int ntiles, TX, TY;
  int fast;                               // 1: FMA build of the push kernels
  int det;                                // 1: fixed-point currents into fj
  FixedJ fj;
};

#ifdef __CUDACC__
// appends a particle to a spill list; flags the host (re-layout due) and
// records an overflow when the list is full
__device__ __forceinline__ void spill_particle(const Spill &S, int *errbits, int ix, int iy, float x, float y,
                                               float ux, float uy, float uz) {
  const int q = atomicAdd(S.cnt, 1);
  *errbits |= ERR_SPILLED;
  if (q < S.cap) store_particle(S.p, q, ix, iy, x, y, ux, uy, uz);
  else *errbits |= ERR_OVERFLOW;
}

__device__ __forceinline__ void spill_particle(const Spill &S, int *errbits, const PRec &r) {
  spill_particle(S, errbits, r.ix, r.iy, r.x, r.y, r.ux, r.uy, r.uz);
}
#endif

// particles
bool tile_supported(int TX, int TY);
cudaError_t launch_push_tiles(const PushLaunch &a, cudaStream_t st);
cudaError_t launch_push_tiles_exact(const PushLaunch &a, cudaStream_t st);
cudaError_t launch_push_tiles_fast(const PushLaunch &a, cudaStream_t st);
cudaError_t launch_push_tiles_exact_det(const PushLaunch &a, cudaStream_t st);
cudaError_t launch_push_tiles_fast_det(const PushLaunch &a, cudaStream_t st);
// sets the shared-memory limit of the deterministic push kernels of one
// tile shape on the current device (outside any stream capture)
cudaError_t prepare_push_tiles_exact_det(int TX, int TY);
cudaError_t prepare_push_tiles_fast_det(int TX, int TY);
// spill push; with det, currents go to fj and the kinetic energy to ekin[0..1]
// read as the two 64-bit fixed-point words of efix_join
cudaError_t launch_push_spill(const float *EB, float *J, const FixedJ &fj, const Grid &G, const Particles &sin,
                              const int *sin_cnt, int sin_cap, const Spill &S, double *ekin, int *err,
                              const PushConst &C, int nblocks, int fast, int det, cudaStream_t st);
#define ZC_SPILL_LAUNCHER(name)                                                                              \
  cudaError_t name(const float *EB, float *J, const FixedJ &fj, const Grid &G, const Particles &sin,          \
                   const int *sin_cnt, int sin_cap, const Spill &S, double *ekin, int *err, const PushConst &C, \
                   int nblocks, cudaStream_t st)
ZC_SPILL_LAUNCHER(launch_push_spill_exact);
ZC_SPILL_LAUNCHER(launch_push_spill_fast);
ZC_SPILL_LAUNCHER(launch_push_spill_exact_det);
ZC_SPILL_LAUNCHER(launch_push_spill_fast_det);
// fixed-point current planes <-> float planes (n values)
cudaError_t launch_fixed_to_float(const unsigned long long *src, float *dst, size_t n, cudaStream_t st);
cudaError_t launch_float_to_fixed(const float *src, unsigned long long *dst, size_t n, cudaStream_t st);
// counting sort of every tile by cell (src -> dst, same offsets): holes
// dropped, np set to the particle count, cell order through tile_slot;
// max_n: the particles a tile stages in shared memory (a tile with more
// takes the rest from global memory; 0: no staging, the sort for runs that
// share the GPU); a timed-out wait on the staging copies sets ERR_TIMEOUT
// in err
cudaError_t launch_cellsort(const Particles &src, const Particles &dst, const int *off, int *np,
                            const LayoutConst &L, int ntiles, int max_n, int *err, cudaStream_t st);
// particles (slots that are not holes) of every tile into cnt
cudaError_t launch_count_valid(const Particles &buf, const int *off, const int *np, int *cnt, int ntiles,
                               cudaStream_t st);
// moves the particles pending in an outbox into their tiles (appended)
cudaError_t launch_settle(const Particles &buf, const TileSet &T, const Outbox &O, const Spill &S, int *err,
                          int ntx, int nty, int mw, cudaStream_t st);
// AoS records (device memory or mapped host memory) -> SoA list; cell_cnt
// (nx * ny counters, or null) receives the particles of every cell
cudaError_t launch_stage_to_list(const void *aos, int n, const Particles &list, int *cell_cnt,
                                 const LayoutConst &L, int *err, cudaStream_t st);
// per tile: cell counts -> first positions of the cells (in place), tile counts
cudaError_t launch_cell_starts(int *cell, int *cnt, const LayoutConst &L, int ntiles, cudaStream_t st);
// list -> tiles in the sorted (lane-run) layout, from the cell starts
cudaError_t launch_scatter_sorted(const Particles &list, int n, const Particles &dst, const int *off,
                                  const int *cnt, int *cell_pos, const LayoutConst &L, cudaStream_t st);
cudaError_t launch_count_list(const Particles &list, const int *n_ptr, int n_cap, int *cnt, const LayoutConst &L,
                              cudaStream_t st);
cudaError_t launch_copy_tiles(const Particles &src, const int *off_old, const int *np_old, const Particles &dst,
                              const int *off_new, int *fill, int ntiles, cudaStream_t st);
cudaError_t launch_scatter_list(const Particles &list, const int *n_ptr, int n_cap, const Particles &dst,
                                const int *off, const int *cap, int *fill, const LayoutConst &L, int *err,
                                cudaStream_t st);
cudaError_t launch_append_list(const Particles &list, int n, const Particles &buf, const TileSet &T,
                               const Spill &S, const LayoutConst &L, int *err, cudaStream_t st);
// a column of cold particles injected after a window move: per row of the
// column, the ppc lattice positions that pass the density test, in the order
// of spec_set_x (em2d/particles.c:159-211, 335-349)
struct ColumnInject {
  int ix, ny, cnt;  // column, rows, particles per cell
  float ux, uy, uz;
  float px[64], py[64];
};
cudaError_t launch_inject_column(const Particles &list, const ColumnInject &C, cudaStream_t st);
cudaError_t launch_gather_aos(const Particles &buf, const int *off, const int *np, const long long *dst_off,
                              int *aos, int ntiles, cudaStream_t st);
cudaError_t launch_list_to_aos(const Particles &list, const int *n_ptr, int n_cap, int *aos, long long d0,
                               cudaStream_t st);
// device-side loading: lattice spacing, per-column inclusion masks (bit a
// of colmask[i]: lattice point a of column i is inside the profile),
// thermal spread and drift, generator key
struct InitConst {
  int ppcx, ppcy;
  float hx, hy;
  float uth[3], ufl[3];
  unsigned seed_lo, seed_hi;
};
cudaError_t launch_init_tiles(const Particles &buf, const int *off, const int *colpts, const unsigned *colmask,
                              const InitConst &I, const LayoutConst &L, int ntiles, cudaStream_t st);
// phase-space density of one species (quantity codes 1 x1, 2 x2, 4 u1,
// 5 u2, 6 u3), added to pha[n1 * n2]
struct PhaConst {
  int q1, q2, n1, n2;
  float x1min, x2min, rdx1, rdx2, dx, dy, q;
};
cudaError_t launch_phasespace(const Particles &buf, const int *off, const int *np, int ntiles, const Particles &spill,
                              const int *spill_cnt, int spill_cap, float *pha, const PhaConst &P, cudaStream_t st);
cudaError_t launch_charge(const Particles &buf, const int *off, const int *np, int ntiles, const Particles &spill,
                          const int *spill_cnt, int spill_cap, float *rho, int nx, int ny, float q, int mw,
                          cudaStream_t st);
// with det, extra[0..1] are the two 64-bit fixed-point words of a kinetic
// energy (efix_join)
cudaError_t launch_sum_energy(const double *tiles, int ntiles, const double *extra, double *out, float q_mq,
                              float dx, float dy, int det, cudaStream_t st);

// fields
struct YeeConst {
  float cxb, cyb;                         // (dt/2)/dx, (dt/2)/dy  (emf.c:507-508)
  float cxe, cye, dt;                     // dt/dx, dt/dy, dt      (emf.c:540-541)
  int mw;                                 // moving window: x guard cells are not periodic
};

cudaError_t launch_aos_to_planes(const float *aos, float *planes, const Grid &G, int ncomp, cudaStream_t st);
cudaError_t launch_planes_to_aos(const float *planes, float *aos, const Grid &G, int ncomp, cudaStream_t st);
cudaError_t launch_fold(float *J, const Grid &G, int mw, cudaStream_t st);
// all filter passes along one axis in one launch
constexpr int kMaxSmoothPasses = 16;
struct SmoothPasses {
  int n;
  float sa[kMaxSmoothPasses], sb[kMaxSmoothPasses];
};
// every x filter pass, then every y pass, out of place (Jin -> Jout)
cudaError_t launch_smooth(const float *Jin, float *Jout, const Grid &G, const SmoothPasses &PX,
                          const SmoothPasses &PY, int mw, cudaStream_t st);
// epart (or null): per-block field-energy partials of the new fields, 6
// doubles a block, yee_blocks(G) blocks.  jzero (or null): a current buffer
// the kernel clears (3 planes).  gc: the guard cells are written as the
// guard-cell update leaves them (k_emf_gc then not needed; nx, ny >= 3)
cudaError_t launch_yee(const CUtensorMap *tm_eb, const CUtensorMap *tm_j, float *EBout, const Grid &G,
                       const YeeConst &Y, int *err, double *epart, float *jzero, bool gc, cudaStream_t st);
int yee_blocks(const Grid &G);
cudaError_t launch_emf_gc(float *EB, const Grid &G, int mw, cudaStream_t st);
cudaError_t launch_ext_add(const float *EB, float *EBp, const float *extE, const float *extB, int Etype, int Btype,
                           float3 E0, float3 B0, const Grid &G, cudaStream_t st);
cudaError_t launch_window_shift(const float *EBin, float *EBout, const Grid &G, cudaStream_t st);
// the kinetic-energy words of up to kEkinRefs species, by value
constexpr int kEkinRefs = 32;
struct EkinRefs {
  const double *p[kEkinRefs];
};
// field energy (emf, 6 values) and the species' kinetic energies (kin) written
// by the device into the given arrays (device or mapped host memory); either
// may be null
cudaError_t launch_energy_direct(const float *EB, const Grid &G, double *partial, int nblocks, float dx, float dy,
                                 const EkinRefs &K, int nsp, double *emf, double *kin, cudaStream_t st);
cudaError_t launch_emf_energy(const float *EB, const Grid &G, double *partial, int nblocks, double *out, float dx,
                              float dy, cudaStream_t st);
// the kinetic-energy sum of one species (what k_sum_energy does)
struct KinSum {
  const double *tiles;   // per-tile partials
  const double *extra;   // spill-list partial (two fixed-point words when det)
  int ntiles, det;
  float q_mq;
};
// appends one row (6 field-energy components, then each species' kinetic
// energy) at hist[*hist_n] and increments *hist_n, unless cap rows exist.
// EB null: the partials are already there (the Yee kernel's).  ks (or null):
// the kinetic sums are made here first, into *ekin[k]
cudaError_t launch_energy_history(const float *EB, const Grid &G, double *partial, int nblocks, double *hist,
                                  int *hist_n, int cap, int cols, double *const *ekin, const KinSum *ks, int nsp,
                                  float dx, float dy, cudaStream_t st);
// dst[k] = *src[k] for k < n (error words of a batch)
cudaError_t launch_gather_words(int *const *src, int n, int *dst, cudaStream_t st);
struct LaserConst {
  int type;
  float start, rise, flat, fall, a0, omega0, polarization, W0, focus, axis;
  float dx, dy;
};
cudaError_t launch_laser(float *EB, const Grid &G, const LaserConst &L, cudaStream_t st);

#ifdef __CUDACC__
// longitudinal envelope of a laser pulse (lon_env, em2d/emf.c:158-186 and
// em1d/emf.c:157-180): sin^2 rise and fall around a flat top, evaluated with
// the double-precision sin on float arguments as the reference does
__device__ inline float laser_env(const LaserConst &L, float z) {
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
#endif

// sets the message returned by zc_last_error() on this thread
void set_error_message(const char *msg);

constexpr int kYeeOX = 32, kYeeOY = 16;   // Yee output tile (buffer cells)
constexpr int kYeeBW = kYeeOX + 8;        // TMA box: 4 columns of halo each side
constexpr int kYeeBH = kYeeOY + 3;

}  // namespace zc
