// zc_adjoint.cu -- the differentiable em2d step: a forward engine with
// per-particle charge weights and its hand-written reverse (adjoint), with
// checkpointed recomputation, in float32 or float64.
//
// The physics is em2d's periodic step (sim_iter, em2d/simulation.c:45-56)
// without smoothing or moving window: staggered bilinear gather
// (interpolate_fld, em2d/particles.c:1029-1071), relativistic Boris push and
// move (particles.c:1145-1207), zigzag current deposit (dep_current_zamb,
// particles.c:773-924) scaled by the particle's weight, Yee b/2, e, b/2
// (yee_b / yee_e, em2d/emf.c:500-562).  Fields are periodic nx x ny planes
// without guard cells; the deposit wraps directly, which is what the
// guard-cell fold of current_update_gc (em2d/current.c:118-159) computes.
//
// The objective is the total field energy after the last step,
// L = sum over E, B components of 0.5 dx dy sum f^2 (emf_get_energy,
// em2d/emf.c:729-750).  Its gradient with respect to the initial state --
// every particle's weight, momenta and position, and the initial E and B --
// comes from one reverse sweep:
//   Yee: the transposed curls (forward differences transpose to negative
//        backward ones on the periodic grid and vice versa);
//   deposit: the transpose of the deposit is a gather of the current's
//        adjoint along the same zigzag segments; its derivative with respect
//        to the start position, the displacement and v_z comes from running
//        the deposit code on 5-way forward-mode dual numbers;
//   push: Boris + move on 9-way dual numbers (momentum, E_p, B_p);
//   gather: its transpose scatters the adjoint of E_p, B_p onto the grid
//        with the same weights; the derivative of the weights with respect
//        to the position comes from 2-way dual numbers.
// The deposit and the gather are piecewise polynomial in the position: the
// gradient is that of the piece the trajectory lies in (kinks where a
// trajectory crosses a cell edge or the half-cell of the staggered gather).
//
// Checkpoints: the state (particles, E, B) is kept every K steps of the
// forward run, which also keeps the pre-step states of its last two
// segments (of its last one when two would take more than 8 GiB); the
// reverse sweep walks those back directly, and recomputes every earlier
// segment of K steps from its checkpoint, keeping its pre-step states, before
// walking it backwards.  A kept step writes its particles straight into the
// next step's slot, so keeping costs only the copies of E and B.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/zpic_cuda.h"
#include "zc_internal.cuh"
#include "zc_kernels.h"

namespace {

// ---------------------------------------------------------------------------
// forward-mode dual numbers
// ---------------------------------------------------------------------------
template <class R, int N>
struct Dual {
  R v;
  R d[N];
  __device__ Dual() {}
  __device__ Dual(R x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = R(0);
  }
};

template <class R, int N>
__device__ __forceinline__ Dual<R, N> seed(R x, int k) {
  Dual<R, N> r(x);
  r.d[k] = R(1);
  return r;
}

#define DUAL_T template <class R, int N>
DUAL_T __device__ __forceinline__ Dual<R, N> operator+(const Dual<R, N> &a, const Dual<R, N> &b) {
  Dual<R, N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator-(const Dual<R, N> &a, const Dual<R, N> &b) {
  Dual<R, N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator-(const Dual<R, N> &a) {
  Dual<R, N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator*(const Dual<R, N> &a, const Dual<R, N> &b) {
  Dual<R, N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator/(const Dual<R, N> &a, const Dual<R, N> &b) {
  Dual<R, N> r;
  r.v = a.v / b.v;
  const R ib = R(1) / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator+(const Dual<R, N> &a, R b) {
  Dual<R, N> r = a;
  r.v += b;
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator+(R a, const Dual<R, N> &b) { return b + a; }
DUAL_T __device__ __forceinline__ Dual<R, N> operator-(const Dual<R, N> &a, R b) {
  Dual<R, N> r = a;
  r.v -= b;
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator-(R a, const Dual<R, N> &b) {
  Dual<R, N> r;
  r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator*(const Dual<R, N> &a, R b) {
  Dual<R, N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator*(R a, const Dual<R, N> &b) { return b * a; }
DUAL_T __device__ __forceinline__ Dual<R, N> operator/(const Dual<R, N> &a, R b) {
  Dual<R, N> r;
  r.v = a.v / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
DUAL_T __device__ __forceinline__ Dual<R, N> operator/(R a, const Dual<R, N> &b) { return Dual<R, N>(a) / b; }
DUAL_T __device__ __forceinline__ Dual<R, N> sqrt_(const Dual<R, N> &a) {
  Dual<R, N> r;
  r.v = sqrt(a.v);
  const R h = R(0.5) / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
#undef DUAL_T

__device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
__device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }
__device__ __forceinline__ float value(float a) { return a; }
__device__ __forceinline__ double value(double a) { return a; }
template <class R, int N>
__device__ __forceinline__ R value(const Dual<R, N> &a) {
  return a.v;
}

// ---------------------------------------------------------------------------
// state and grids
// ---------------------------------------------------------------------------
__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// 3 planes [c][j][i], periodic in y.  Periodic runs: nx columns, periodic
// in x.  Moving window: nx + 3 columns holding cells -1 .. nx+1 (the
// reference's x guard cells, em2d/emf.c:59-89), not periodic in x.
template <class R>
struct Planes {
  R *f;
  int nx, ny, mw;
  __device__ __forceinline__ int pitch() const { return mw ? nx + 3 : nx; }
  __device__ __forceinline__ size_t at(int c, int i, int j) const {
    const int pt = pitch();
    return (size_t)c * pt * ny + (size_t)wrap(j, ny) * pt + (mw ? i + 1 : wrap(i, nx));
  }
  __device__ __forceinline__ R operator()(int c, int i, int j) const { return f[at(c, i, j)]; }
};

template <class R>
struct State {
  int *ix, *iy, *alive;  // alive: 0 once the particle left through an absorbing x edge
  R *x, *y, *ux, *uy, *uz;
};

template <class R>
struct Params {
  int nx, ny, np;
  R tem, dt_dx, dt_dy, q, qnx, qny;  // qnx = q dx / dt (per unit weight)
  int mw;                             // moving window: absorbing x edges, window shifts
  int shift;                          // this step shifts the window
  int n;                              // step index (particles are born at their birth step)
};

// a particle takes part in step P.n
template <class R>
__device__ __forceinline__ bool active(const State<R> &s, const int *birth, int p, const Params<R> &P) {
  return s.alive[p] && (!birth || birth[p] <= P.n);
}

// staggered bilinear gather (interpolate_fld): weights of type T, field
// samples of type R
template <class R, class T>
__device__ __forceinline__ T lerp2(const Planes<R> &g, int c, int a, int b, const T &wa, const T &wb) {
  return (g(c, a, b) * (R(1) - wa) + g(c, a + 1, b) * wa) * (R(1) - wb) +
         (g(c, a, b + 1) * (R(1) - wa) + g(c, a + 1, b + 1) * wa) * wb;
}

template <class R, class T>
__device__ __forceinline__ void gather(const Planes<R> &E, const Planes<R> &B, int i, int j, const T &x, const T &y,
                                       T f[6]) {
  const bool lx = value(x) < R(0.5), ly = value(y) < R(0.5);
  const int ih = i + (lx ? -1 : 0), jh = j + (ly ? -1 : 0);
  const T w1h = x + (lx ? R(0.5) : R(-0.5));
  const T w2h = y + (ly ? R(0.5) : R(-0.5));
  f[0] = lerp2(E, 0, ih, j, w1h, y);
  f[1] = lerp2(E, 1, i, jh, x, w2h);
  f[2] = lerp2(E, 2, i, j, x, y);
  f[3] = lerp2(B, 0, i, jh, x, w2h);
  f[4] = lerp2(B, 1, ih, j, w1h, y);
  f[5] = lerp2(B, 2, ih, jh, w1h, w2h);
}

// transpose of the gather: adds a[c] times the weights of sample c to the
// grids (ga for E, gb for B)
template <class R>
__device__ __forceinline__ void scatter_add(R *ga, R *gb, const Planes<R> &shape, int i, int j, R x, R y,
                                            const R a[6]) {
  const bool lx = x < R(0.5), ly = y < R(0.5);
  const int ih = i + (lx ? -1 : 0), jh = j + (ly ? -1 : 0);
  const R w1h = x + (lx ? R(0.5) : R(-0.5));
  const R w2h = y + (ly ? R(0.5) : R(-0.5));
  auto put = [&](R *g, int c, int a0, int b0, R wa, R wb, R v) {
    if (v == R(0)) return;
    atomicAdd(&g[shape.at(c, a0, b0)], v * (R(1) - wa) * (R(1) - wb));
    atomicAdd(&g[shape.at(c, a0 + 1, b0)], v * wa * (R(1) - wb));
    atomicAdd(&g[shape.at(c, a0, b0 + 1)], v * (R(1) - wa) * wb);
    atomicAdd(&g[shape.at(c, a0 + 1, b0 + 1)], v * wa * wb);
  };
  put(ga, 0, ih, j, w1h, y, a[0]);
  put(ga, 1, i, jh, x, w2h, a[1]);
  put(ga, 2, i, j, x, y, a[2]);
  put(gb, 0, i, jh, x, w2h, a[3]);
  put(gb, 1, ih, j, w1h, y, a[4]);
  put(gb, 2, ih, jh, w1h, w2h, a[5]);
}

// Boris push and move (particles.c:1145-1207): momentum, E_p, B_p in;
// new momentum, displacement (cells) and q v_z per unit weight out
template <class R, class T>
__device__ __forceinline__ void boris(const T u[3], const T e_in[3], const T b_in[3], const Params<R> &P, T uo[3],
                                      T &mx, T &my, T &qvz) {
  const T ex = e_in[0] * P.tem, ey = e_in[1] * P.tem, ez = e_in[2] * P.tem;
  T tx = u[0] + ex, ty = u[1] + ey, tz = u[2] + ez;
  const T u2 = tx * tx + ty * ty + tz * tz;
  const T g = sqrt_(R(1) + u2);
  const T tg = P.tem / g;
  T bx = b_in[0] * tg, by = b_in[1] * tg, bz = b_in[2] * tg;
  const T s2 = R(2) / (R(1) + bx * bx + by * by + bz * bz);
  const T vx = tx + ty * bz - tz * by;
  const T vy = ty + tz * bx - tx * bz;
  const T vz = tz + tx * by - ty * bx;
  bx = bx * s2;
  by = by * s2;
  bz = bz * s2;
  tx = tx + (vy * bz - vz * by);
  ty = ty + (vz * bx - vx * bz);
  tz = tz + (vx * by - vy * bx);
  uo[0] = tx + ex;
  uo[1] = ty + ey;
  uo[2] = tz + ez;
  const T rg = R(1) / sqrt_(R(1) + uo[0] * uo[0] + uo[1] * uo[1] + uo[2] * uo[2]);
  mx = P.dt_dx * rg * uo[0];
  my = P.dt_dy * rg * uo[1];
  qvz = P.q * uo[2] * rg;
}

// kinetic-energy term utsq / (gamma + 1) of the time-centred momentum
template <class R>
__device__ __forceinline__ R kinetic(const R u[3], const R e_in[3], const Params<R> &P) {
  const R tx = u[0] + e_in[0] * P.tem, ty = u[1] + e_in[1] * P.tem, tz = u[2] + e_in[2] * P.tem;
  const R u2 = tx * tx + ty * ty + tz * tz;
  return u2 / (sqrt_(R(1) + u2) + R(1));
}

// reverse of boris(): cotangents of (new momentum, mx, my, q v_z) in, of
// (momentum, E_p, B_p) out; the forward intermediates are recomputed
template <class R>
struct V3 {
  R x, y, z;
};
template <class R>
__device__ __forceinline__ V3<R> cross(const V3<R> &a, const V3<R> &b) {
  return V3<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
__device__ __forceinline__ R dot(const V3<R> &a, const V3<R> &b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class R>
__device__ __forceinline__ V3<R> axpy(R a, const V3<R> &x, const V3<R> &y) {  // a x + y
  return V3<R>{a * x.x + y.x, a * x.y + y.y, a * x.z + y.z};
}

template <class R>
__device__ __forceinline__ void boris_vjp(const R u_in[3], const R e_in[3], const R b_in[3], const Params<R> &P,
                                          const R lu_out[3], R lmx, R lmy, R lqvz, R lu[3], R le[3], R lb[3]) {
  // forward
  const V3<R> e{e_in[0] * P.tem, e_in[1] * P.tem, e_in[2] * P.tem};
  const V3<R> t0{u_in[0] + e.x, u_in[1] + e.y, u_in[2] + e.z};
  const R u2 = dot(t0, t0);
  const R g = sqrt_(R(1) + u2);
  const R tg = P.tem / g;
  const V3<R> B{b_in[0], b_in[1], b_in[2]};
  const V3<R> b{B.x * tg, B.y * tg, B.z * tg};
  const R s2 = R(2) / (R(1) + dot(b, b));
  const V3<R> v = axpy(R(1), t0, cross(t0, b));
  const V3<R> b2{b.x * s2, b.y * s2, b.z * s2};
  const V3<R> t1 = axpy(R(1), t0, cross(v, b2));
  const V3<R> uo = axpy(R(1), t1, e);
  const R rg = R(1) / sqrt_(R(1) + dot(uo, uo));
  // reverse
  V3<R> luo{lu_out[0] + P.dt_dx * rg * lmx, lu_out[1] + P.dt_dy * rg * lmy, lu_out[2] + P.q * rg * lqvz};
  const R lrg = P.dt_dx * uo.x * lmx + P.dt_dy * uo.y * lmy + P.q * uo.z * lqvz;
  luo = axpy(-rg * rg * rg * lrg, uo, luo);
  // uo = t1 + e ; t1 = t0 + v x b2
  V3<R> le_ = luo;
  V3<R> lt0 = luo;
  const V3<R> lv = cross(b2, luo);
  const V3<R> lb2 = cross(luo, v);
  // b2 = b s2
  V3<R> lbv{s2 * lb2.x, s2 * lb2.y, s2 * lb2.z};
  const R ls2 = dot(b, lb2);
  // v = t0 + t0 x b
  lt0 = axpy(R(1), lv, lt0);
  lt0 = axpy(R(1), cross(b, lv), lt0);
  lbv = axpy(R(1), cross(lv, t0), lbv);
  // s2 = 2 / (1 + |b|^2)
  lbv = axpy(-s2 * s2 * ls2, b, lbv);
  // b = B tg
  const V3<R> lB{tg * lbv.x, tg * lbv.y, tg * lbv.z};
  const R ltg = dot(B, lbv);
  // tg = tem / g ; g = sqrt(1 + u2) ; u2 = |t0|^2
  const R lg = -tg / g * ltg;
  const R lu2 = lg / (R(2) * g);
  lt0 = axpy(R(2) * lu2, t0, lt0);
  // t0 = u + e ; e = E tem
  le_ = axpy(R(1), lt0, le_);
  lu[0] = lt0.x;
  lu[1] = lt0.y;
  lu[2] = lt0.z;
  le[0] = P.tem * le_.x;
  le[1] = P.tem * le_.y;
  le[2] = P.tem * le_.z;
  lb[0] = lB.x;
  lb[1] = lB.y;
  lb[2] = lB.z;
}

// the 8 contributions of one straight segment inside one cell
// (particles.c:886-922), per unit weight
template <class R, class T, class Sink>
__device__ __forceinline__ void segment(Sink &sink, int ix, int iy, const T &x0, const T &x1, const T &y0,
                                        const T &y1, const T &dx, const T &dy, const T &qvz, const Params<R> &P) {
  const T s0x0 = R(1) - x0, s0x1 = x0, s1x0 = R(1) - x1, s1x1 = x1;
  const T s0y0 = R(1) - y0, s0y1 = y0, s1y0 = R(1) - y1, s1y1 = y1;
  const T jx = dx * P.qnx, jy = dy * P.qny;
  sink.add(0, ix, iy, jx * (R(0.5) * (s0y0 + s1y0)));
  sink.add(0, ix, iy + 1, jx * (R(0.5) * (s0y1 + s1y1)));
  sink.add(1, ix, iy, jy * (R(0.5) * (s0x0 + s1x0)));
  sink.add(1, ix + 1, iy, jy * (R(0.5) * (s0x1 + s1x1)));
  sink.add(2, ix, iy, qvz * (s0x0 * s0y0 + s1x0 * s1y0 + (s0x0 * s1y0 - s1x0 * s0y0) / R(2)));
  sink.add(2, ix + 1, iy, qvz * (s0x1 * s0y0 + s1x1 * s1y0 + (s0x1 * s1y0 - s1x1 * s0y0) / R(2)));
  sink.add(2, ix, iy + 1, qvz * (s0x0 * s0y1 + s1x0 * s1y1 + (s0x0 * s1y1 - s1x0 * s0y1) / R(2)));
  sink.add(2, ix + 1, iy + 1, qvz * (s0x1 * s0y1 + s1x1 * s1y1 + (s0x1 * s1y1 - s1x1 * s0y1) / R(2)));
}

template <class T>
struct SegT {
  T x0, x1, y0, y1, dx, dy, qvz;
  int ix, iy;
};

// splits segment a at its y cell edge: a keeps the part before the edge, the
// returned segment holds the rest (particles.c:842-871)
template <class R, class T>
__device__ __forceinline__ SegT<T> split_y(SegT<T> &a, int dj) {
  const R yb = (dj == 1) ? R(1) : R(0);
  const T f = (a.y1 - yb) / a.dy;
  const T xc = a.x0 + a.dx * (R(1) - f);
  SegT<T> n;
  n.y0 = T(R(1) - yb);
  n.y1 = a.y1 - R(dj);
  n.dy = a.dy * f;
  n.iy = a.iy + dj;
  n.x0 = xc;
  n.x1 = a.x1;
  n.dx = a.dx * f;
  n.ix = a.ix;
  n.qvz = a.qvz * f;
  a.y1 = T(yb);
  a.dy = a.dy * (R(1) - f);
  a.dx = a.dx * (R(1) - f);
  a.x1 = xc;
  a.qvz = a.qvz * (R(1) - f);
  return n;
}

template <class R, class T, class Sink>
__device__ __forceinline__ void deposit_seg(Sink &sink, const SegT<T> &s, const Params<R> &P) {
  segment(sink, s.ix, s.iy, s.x0, s.x1, s.y0, s.y1, s.dx, s.dy, s.qvz, P);
}

// zigzag split of a motion into at most 3 segments (particles.c:773-879)
template <class R, class T, class Sink>
__device__ __forceinline__ void zigzag(Sink &sink, int ix, int iy, const T &x0, const T &y0, const T &dx,
                                       const T &dy, const T &qvz, const Params<R> &P) {
  SegT<T> a;
  a.x0 = x0;
  a.y0 = y0;
  a.dx = dx;
  a.dy = dy;
  a.x1 = x0 + dx;
  a.y1 = y0 + dy;
  a.qvz = qvz * R(0.5);
  a.ix = ix;
  a.iy = iy;
  const int di = (value(a.x1) >= R(1)) - (value(a.x1) < R(0));
  const int dj = (value(a.y1) >= R(1)) - (value(a.y1) < R(0));
  if (di != 0) {
    const R xb = (di == 1) ? R(1) : R(0);
    const T f = (a.x1 - xb) / dx;
    const T yc = y0 + dy * (R(1) - f);
    SegT<T> b;
    b.x0 = T(R(1) - xb);
    b.x1 = a.x1 - R(di);
    b.dx = dx * f;
    b.ix = ix + di;
    b.y0 = yc;
    b.y1 = a.y1;
    b.dy = dy * f;
    b.iy = iy;
    b.qvz = a.qvz * f;
    a.x1 = T(xb);
    a.dx = a.dx * (R(1) - f);
    a.dy = a.dy * (R(1) - f);
    a.y1 = yc;
    a.qvz = a.qvz * (R(1) - f);
    if (dj != 0) {
      if (value(a.y1) < R(0) || value(a.y1) >= R(1)) {
        // the first piece crosses the y edge; the x tail lies past it
        const SegT<T> c = split_y<R, T>(a, dj);
        b.y0 = b.y0 - R(dj);
        b.y1 = b.y1 - R(dj);
        b.iy += dj;
        deposit_seg(sink, c, P);
      } else {
        const SegT<T> c = split_y<R, T>(b, dj);
        deposit_seg(sink, c, P);
      }
    }
    deposit_seg(sink, b, P);
  } else if (dj != 0) {
    const SegT<T> c = split_y<R, T>(a, dj);
    deposit_seg(sink, c, P);
  }
  deposit_seg(sink, a, P);
}

// ---------------------------------------------------------------------------
// sinks of the deposit
// ---------------------------------------------------------------------------
template <class R>
struct DepositSink {  // forward: J += w * contribution
  Planes<R> J;
  R w;
  __device__ __forceinline__ void add(int c, int i, int j, R v) const { atomicAdd(&J.f[J.at(c, i, j)], w * v); }
};

// reverse: sums of lambda_J times the contributions (per unit weight), the
// x and y components apart from z (the deposit runs with q v_z = 1: the z
// contributions are linear in it)
template <class R, int N>
struct AdjointSink {
  Planes<R> lamJ;
  Dual<R, N> axy, az;
  __device__ __forceinline__ void add(int c, int i, int j, const Dual<R, N> &v) {
    const R l = lamJ(c, i, j);
    Dual<R, N> &a = (c == 2) ? az : axy;
    a.v += l * v.v;
#pragma unroll
    for (int k = 0; k < N; ++k) a.d[k] += l * v.d[k];
  }
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
template <class R>
__global__ void k_adj_push(State<R> s, State<R> o, const R *w, const int *birth, Planes<R> E, Planes<R> B,
                           Planes<R> J, double *ekin, Params<R> P) {
  double ek = 0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.np; p += gridDim.x * blockDim.x) {
    if (!active(s, birth, p, P)) {  // not born yet or gone: carried over unchanged
      o.ix[p] = s.ix[p];
      o.iy[p] = s.iy[p];
      o.alive[p] = s.alive[p];
      o.x[p] = s.x[p];
      o.y[p] = s.y[p];
      o.ux[p] = s.ux[p];
      o.uy[p] = s.uy[p];
      o.uz[p] = s.uz[p];
      continue;
    }
    const int ix = s.ix[p], iy = s.iy[p];
    const R x = s.x[p], y = s.y[p];
    const R u[3] = {s.ux[p], s.uy[p], s.uz[p]};
    R f[6];
    gather<R, R>(E, B, ix, iy, x, y, f);
    ek += (double)w[p] * (double)kinetic(u, f, P);
    R uo[3], mx, my, qvz;
    boris<R, R>(u, f, f + 3, P, uo, mx, my, qvz);
    DepositSink<R> sink{J, w[p]};
    zigzag<R, R>(sink, ix, iy, x, y, mx, my, qvz, P);
    R x1 = x + mx, y1 = y + my;
    const int di = (x1 >= R(1)) - (x1 < R(0)), dj = (y1 >= R(1)) - (y1 < R(0));
    x1 -= R(di);
    y1 -= R(dj);
    // periodic, or (moving window) the shift and the absorbing x edges
    // (particles.c:1234-1259, spec_move_window particles.c:619-640)
    const int nix = P.mw ? ix + di - P.shift : wrap(ix + di, P.nx);
    o.ix[p] = nix;
    o.alive[p] = P.mw ? (nix >= 0 && nix < P.nx) : 1;
    o.iy[p] = wrap(iy + dj, P.ny);
    o.x[p] = x1;
    o.y[p] = y1;
    o.ux[p] = uo[0];
    o.uy[p] = uo[1];
    o.uz[p] = uo[2];
  }
  if (ekin && ek != 0.0) atomicAdd(ekin, ek);
}

// the contributions of a motion that stays in its cell: one segment
template <class R, class T, class Sink>
__device__ __forceinline__ void single_segment(Sink &sink, int ix, int iy, const T &x0, const T &y0, const T &dx,
                                               const T &dy, const T &qvz, const Params<R> &P) {
  segment(sink, ix, iy, x0, x0 + dx, y0, y0 + dy, dx, dy, qvz * R(0.5), P);
}

// Reverse of one particle step: lam (x, y, ux, uy, uz) of the particle after
// the step in, before the step out (in place); lamE / lamB receive the
// transpose of the gather; dw the weight's derivative.  FULL handles any
// motion (up to three zigzag segments); the light variant only motions
// that stay in their cell and returns false for the others untouched.
template <class R, bool FULL>
__device__ __forceinline__ bool reverse_particle(int p, const State<R> &s, const R *w, const int *birth,
                                                 const Planes<R> &E, const Planes<R> &B, const Planes<R> &lamJ,
                                                 const State<R> &lam, R *lamE, R *lamB, R *dw, const Params<R> &P) {
  if (!active(s, birth, p, P)) return true;  // took no part in this step
  const int ix = s.ix[p], iy = s.iy[p];
  const R x = s.x[p], y = s.y[p];
  const R u[3] = {s.ux[p], s.uy[p], s.uz[p]};
  // 1. gather with d/dx, d/dy
  Dual<R, 2> fd[6];
  gather<R, Dual<R, 2>>(E, B, ix, iy, seed<R, 2>(x, 0), seed<R, 2>(y, 1), fd);
  R f[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) f[c] = fd[c].v;
  // 2. Boris + move (values)
  R uo[3], mx, my, qvz;
  boris<R, R>(u, f, f + 3, P, uo, mx, my, qvz);
  // 3. deposit with d/d(x, y, mx, my); linear in q v_z
  AdjointSink<R, 4> sink{lamJ, Dual<R, 4>(R(0)), Dual<R, 4>(R(0))};
  if constexpr (FULL) {
    zigzag<R, Dual<R, 4>>(sink, ix, iy, seed<R, 4>(x, 0), seed<R, 4>(y, 1), seed<R, 4>(mx, 2), seed<R, 4>(my, 3),
                          Dual<R, 4>(R(1)), P);
  } else {
    const R x1 = x + mx, y1 = y + my;
    if (x1 >= R(1) || x1 < R(0) || y1 >= R(1) || y1 < R(0)) return false;
    single_segment<R, Dual<R, 4>>(sink, ix, iy, seed<R, 4>(x, 0), seed<R, 4>(y, 1), seed<R, 4>(mx, 2),
                                  seed<R, 4>(my, 3), Dual<R, 4>(R(1)), P);
  }
  const R wp = w[p];
  dw[p] += sink.axy.v + qvz * sink.az.v;
  R gdep[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) gdep[k] = wp * (sink.axy.d[k] + qvz * sink.az.d[k]);
  // 4. cotangents of the Boris outputs, then its reverse
  const R lx1 = lam.x[p], ly1 = lam.y[p];
  const R lu1[3] = {lam.ux[p], lam.uy[p], lam.uz[p]};
  R lu0[3], lef[3], lbf[3];
  boris_vjp<R>(u, f, f + 3, P, lu1, lx1 + gdep[2], ly1 + gdep[3], wp * sink.az.v, lu0, lef, lbf);
  // 5. position: direct (x1 = x + mx - di), deposit, and the gather weights
  const R l6[6] = {lef[0], lef[1], lef[2], lbf[0], lbf[1], lbf[2]};
  R lx = lx1 + gdep[0], ly = ly1 + gdep[1];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    lx += l6[c] * fd[c].d[0];
    ly += l6[c] * fd[c].d[1];
  }
  lam.x[p] = lx;
  lam.y[p] = ly;
  lam.ux[p] = lu0[0];
  lam.uy[p] = lu0[1];
  lam.uz[p] = lu0[2];
  // 6. transpose of the gather
  scatter_add(lamE, lamB, E, ix, iy, x, y, l6);
  return true;
}

// the particles whose motion stays in its cell (most of them); the others
// are listed for k_adj_push_rev_cross
template <class R>
__global__ void __launch_bounds__(128) k_adj_push_rev(State<R> s, const R *w, const int *birth, Planes<R> E,
                                                      Planes<R> B, Planes<R> lamJ, State<R> lam, R *lamE, R *lamB,
                                                      R *dw, int *cross, int *ncross, Params<R> P) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.np; p += gridDim.x * blockDim.x)
    if (!reverse_particle<R, false>(p, s, w, birth, E, B, lamJ, lam, lamE, lamB, dw, P))
      cross[atomicAdd(ncross, 1)] = p;
}

// the listed cell-crossing particles
template <class R>
__global__ void __launch_bounds__(128) k_adj_push_rev_cross(State<R> s, const R *w, const int *birth, Planes<R> E,
                                                            Planes<R> B, Planes<R> lamJ, State<R> lam, R *lamE,
                                                            R *lamB, R *dw, const int *cross, const int *ncross,
                                                            Params<R> P) {
  const int n = *ncross;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    reverse_particle<R, true>(cross[k], s, w, birth, E, B, lamJ, lam, lamE, lamB, dw, P);
}

// B -= c curl E  (yee_b with c = dt/2)
template <class R>
__global__ void k_adj_yee_b(const R *E, R *B, int nx, int ny, R cx, R cy) {
  const size_t pl = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const int ip = wrap(i + 1, nx), jp = wrap(j + 1, ny);
    const R *Ex = E, *Ey = E + pl, *Ez = E + 2 * pl;
    B[k] += -cy * (Ez[(size_t)jp * nx + i] - Ez[k]);
    B[pl + k] += cx * (Ez[(size_t)j * nx + ip] - Ez[k]);
    B[2 * pl + k] += -cx * (Ey[(size_t)j * nx + ip] - Ey[k]) + cy * (Ex[(size_t)jp * nx + i] - Ex[k]);
  }
}

// E += dt curl B - dt J  (yee_e)
template <class R>
__global__ void k_adj_yee_e(R *E, const R *B, const R *J, int nx, int ny, R cx, R cy, R dt) {
  const size_t pl = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const int im = wrap(i - 1, nx), jm = wrap(j - 1, ny);
    const R *Bx = B, *By = B + pl, *Bz = B + 2 * pl;
    E[k] += cy * (Bz[k] - Bz[(size_t)jm * nx + i]) - dt * J[k];
    E[pl + k] += -cx * (Bz[k] - Bz[(size_t)j * nx + im]) - dt * J[pl + k];
    E[2 * pl + k] += cx * (By[k] - By[(size_t)j * nx + im]) - cy * (Bx[k] - Bx[(size_t)jm * nx + i]) - dt * J[2 * pl + k];
  }
}

// transpose of k_adj_yee_b: lamE += transpose(-c curl) lamB
template <class R>
__global__ void k_adj_yee_b_T(const R *lB, R *lE, int nx, int ny, R cx, R cy) {
  const size_t pl = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const int im = wrap(i - 1, nx), jm = wrap(j - 1, ny);
    const R *ax = lB, *ay = lB + pl, *az = lB + 2 * pl;
    // B.x(i,j) -= cy (Ez(i,j+1) - Ez(i,j)); B.y += cx (Ez(i+1,j) - Ez(i,j));
    // B.z += -cx (Ey(i+1,j) - Ey(i,j)) + cy (Ex(i,j+1) - Ex(i,j))
    lE[k] += cy * (az[(size_t)jm * nx + i] - az[k]);
    lE[pl + k] += -cx * (az[(size_t)j * nx + im] - az[k]);
    lE[2 * pl + k] += -cy * (ax[(size_t)jm * nx + i] - ax[k]) + cx * (ay[(size_t)j * nx + im] - ay[k]);
  }
}

// transpose of k_adj_yee_e: lamB += transpose(dt curl) lamE, lamJ = -dt lamE
template <class R>
__global__ void k_adj_yee_e_T(const R *lE, R *lB, R *lJ, int nx, int ny, R cx, R cy, R dt) {
  const size_t pl = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const int ip = wrap(i + 1, nx), jp = wrap(j + 1, ny);
    const R *ax = lE, *ay = lE + pl, *az = lE + 2 * pl;
    // E.x += cy (Bz(i,j) - Bz(i,j-1)); E.y += -cx (Bz(i,j) - Bz(i-1,j));
    // E.z += cx (By(i,j) - By(i-1,j)) - cy (Bx(i,j) - Bx(i,j-1))
    lB[k] += -cy * (az[k] - az[(size_t)jp * nx + i]);
    lB[pl + k] += cx * (az[k] - az[(size_t)j * nx + ip]);
    lB[2 * pl + k] += cy * (ax[k] - ax[(size_t)jp * nx + i]) - cx * (ay[k] - ay[(size_t)j * nx + ip]);
    lJ[k] = -dt * ax[k];
    lJ[pl + k] = -dt * ay[k];
    lJ[2 * pl + k] = -dt * az[k];
  }
}

// ---------------------------------------------------------------------------
// moving window: planes of nx + 3 columns (cells -1 .. nx+1), periodic in y
// ---------------------------------------------------------------------------
// yee_b over the reference's range, cells -1 .. nx (em2d/emf.c:500-522)
template <class R>
__global__ void k_adj_yee_b_mw(const R *E, R *B, int nx, int ny, R cx, R cy) {
  const int pt = nx + 3;
  const size_t pl = (size_t)pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt), j = (int)(k / pt);  // buffer column b = cell b - 1
    if (b > nx + 1) continue;
    const size_t kp = (size_t)wrap(j + 1, ny) * pt + b, kr = k + 1;
    const R *Ex = E, *Ey = E + pl, *Ez = E + 2 * pl;
    B[k] += -cy * (Ez[kp] - Ez[k]);
    B[pl + k] += cx * (Ez[kr] - Ez[k]);
    B[2 * pl + k] += -cx * (Ey[kr] - Ey[k]) + cy * (Ex[kp] - Ex[k]);
  }
}

// yee_e over the reference's range, cells 0 .. nx+1 (em2d/emf.c:531-562)
template <class R>
__global__ void k_adj_yee_e_mw(R *E, const R *B, const R *J, int nx, int ny, R cx, R cy, R dt) {
  const int pt = nx + 3;
  const size_t pl = (size_t)pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt), j = (int)(k / pt);
    if (b < 1) continue;
    const size_t km = (size_t)wrap(j - 1, ny) * pt + b, kl = k - 1;
    const R *Bx = B, *By = B + pl, *Bz = B + 2 * pl;
    E[k] += cy * (Bz[k] - Bz[km]) - dt * J[k];
    E[pl + k] += -cx * (Bz[k] - Bz[kl]) - dt * J[pl + k];
    E[2 * pl + k] += cx * (By[k] - By[kl]) - cy * (Bx[k] - Bx[km]) - dt * J[2 * pl + k];
  }
}

// transpose of k_adj_yee_b_mw: lamE += transpose(-c curl) lamB
template <class R>
__global__ void k_adj_yee_b_T_mw(const R *lB, R *lE, int nx, int ny, R cx, R cy) {
  const int pt = nx + 3;
  const size_t pl = (size_t)pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt), j = (int)(k / pt);
    const bool in = b <= nx + 1, inl = b >= 1 && b - 1 <= nx + 1;  // cell and its left neighbour updated
    const size_t km = (size_t)wrap(j - 1, ny) * pt + b;
    const R *ax = lB, *ay = lB + pl, *az = lB + 2 * pl;
    R ex = 0, ey = 0, ez = 0;
    if (in) {
      ex += cy * (az[km] - az[k]);
      ey += cx * az[k];
      ez += cy * (ax[k] - ax[km]) - cx * ay[k];
    }
    if (inl) {
      ey += -cx * az[k - 1];
      ez += cx * ay[k - 1];
    }
    lE[k] += ex;
    lE[pl + k] += ey;
    lE[2 * pl + k] += ez;
  }
}

// transpose of k_adj_yee_e_mw: lamB += transpose(dt curl) lamE, lamJ = -dt lamE
template <class R>
__global__ void k_adj_yee_e_T_mw(const R *lE, R *lB, R *lJ, int nx, int ny, R cx, R cy, R dt) {
  const int pt = nx + 3;
  const size_t pl = (size_t)pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt), j = (int)(k / pt);
    const bool in = b >= 1, inr = b + 1 <= nx + 2;  // cell and its right neighbour updated
    const size_t kp = (size_t)wrap(j + 1, ny) * pt + b;
    const R *ax = lE, *ay = lE + pl, *az = lE + 2 * pl;
    R bx = 0, by = 0, bz = 0;
    if (in) {
      bz += cy * (ax[k] - ax[kp]) - cx * ay[k];
      by += cx * az[k];
      bx += -cy * (az[k] - az[kp]);
    }
    if (inr) {
      bz += cx * ay[k + 1];
      by += -cx * az[k + 1];
    }
    lB[k] += bx;
    lB[pl + k] += by;
    lB[2 * pl + k] += bz;
    lJ[k] = in ? -dt * ax[k] : R(0);
    lJ[pl + k] = in ? -dt * ay[k] : R(0);
    lJ[2 * pl + k] = in ? -dt * az[k] : R(0);
  }
}

// window shift (emf_move_window, em2d/emf.c:648-675): cells -1 .. nx-2 take
// their right neighbour, cells nx-1 .. nx+1 are zeroed; out of place
template <class R>
__global__ void k_adj_shift(const R *in, R *out, int nx, size_t n) {
  const int pt = nx + 3;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt);
    out[k] = (b < nx) ? in[k + 1] : R(0);
  }
}

// its transpose
template <class R>
__global__ void k_adj_shift_T(const R *lout, R *lin, int nx, size_t n) {
  const int pt = nx + 3;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt);
    lin[k] = (b >= 1 && b - 1 < nx) ? lout[k - 1] : R(0);
  }
}

// one [sa, sb, sa] filter pass along x (kernel_x, em2d/current.c:316-354),
// out of place: periodic runs filter every cell periodically; with a moving
// window the interior cells 0 .. nx-1 are filtered and the guard cells kept
template <class R>
__global__ void k_adj_smooth_x(const R *in, R *out, int nx, int ny, int mw, R sa, R sb) {
  const int pt = mw ? nx + 3 : nx;
  const size_t n = (size_t)3 * pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt);
    const size_t row = k - b;
    if (mw) {
      out[k] = (b >= 1 && b <= nx) ? sa * in[k - 1] + sb * in[k] + sa * in[k + 1] : in[k];
    } else {
      out[k] = sa * in[row + wrap(b - 1, nx)] + sb * in[k] + sa * in[row + wrap(b + 1, nx)];
    }
  }
}

// its transpose
template <class R>
__global__ void k_adj_smooth_x_T(const R *lout, R *lin, int nx, int ny, int mw, R sa, R sb) {
  const int pt = mw ? nx + 3 : nx;
  const size_t n = (size_t)3 * pt * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(k % pt);
    const size_t row = k - b;
    if (mw) {
      auto inner = [&](int c) { return c >= 1 && c <= nx; };
      R v = inner(b) ? sb * lout[k] : lout[k];
      if (b >= 1 && inner(b - 1)) v += sa * lout[k - 1];
      if (b + 1 < pt && inner(b + 1)) v += sa * lout[k + 1];
      lin[k] = v;
    } else {
      lin[k] = sa * lout[row + wrap(b - 1, nx)] + sb * lout[k] + sa * lout[row + wrap(b + 1, nx)];
    }
  }
}

// objective terms of the interior cells: 1 = Ex on row `row`, cells
// i0 .. i1-1 (sum Ex^2 dx),
// 0 = every component (the field energy); writes the adjoint seed and adds
// the objective's sum of squares to *acc
template <class R>
__global__ void k_adj_objective(const R *E, const R *B, R *lE, R *lB, int nx, int ny, int mw, int kind, int row,
                                int i0, int i1, R seed, double *acc) {
  const int pt = mw ? nx + 3 : nx;
  const size_t pl = (size_t)pt * ny;
  __shared__ double sred[8];
  double s = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < 6 * pl; k += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(k / pl);
    const size_t kk = k - (size_t)c * pl;
    const int b = (int)(kk % pt), j = (int)(kk / pt);
    const bool interior = !mw || (b >= 1 && b <= nx);
    const int i = mw ? b - 1 : b;  // cell index
    const bool used = interior && (kind == 0 || (c == 0 && j == row && i >= i0 && i < i1));
    const R f = (c < 3) ? E[k] : B[k - 3 * pl];
    if (used) s += (double)f * (double)f;
    R *l = (c < 3) ? lE + k : lB + (k - 3 * pl);
    if (lE) *l = used ? seed * f : R(0);
  }
  s = zc::block_sum_double<256>(s, sred);
  if (threadIdx.x == 0 && acc) atomicAdd(acc, s);
}

// sum of squares of n values (field energy), double accumulation
template <class R>
__global__ void k_adj_sumsq(const R *f, size_t n, double *out) {
  __shared__ double sred[8];
  double s = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    s += (double)f[k] * (double)f[k];
  s = zc::block_sum_double<256>(s, sred);
  if (threadIdx.x == 0) atomicAdd(out, s);
}

template <class R>
__global__ void k_adj_scale(const R *src, R *dst, size_t n, R a) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = a * src[k];
}

template <class R>
__global__ void k_to_double(const R *src, double *dst, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = (double)src[k];
}

template <class R>
__global__ void k_from_double(const double *src, R *dst, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    dst[k] = (R)src[k];
}

int grid_for(size_t n, int per = 256) { return (int)std::max<size_t>(1, std::min<size_t>((n + per - 1) / per, 152 * 8)); }

zc_status afail(zc_status s, const char *msg) {
  zc::set_error_message(msg);
  return s;
}

#define ACK(call)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) {                                                                        \
      char b_[256];                                                                                 \
      snprintf(b_, sizeof b_, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return afail(ZC_ECUDA, b_);                                                                   \
    }                                                                                               \
  } while (0)

// ---------------------------------------------------------------------------
// host engine
// ---------------------------------------------------------------------------
#define TRY_(c)                   \
  do {                            \
    zc_status s_ = (c);           \
    if (s_ != ZC_OK) return s_;   \
  } while (0)

struct EngineBase {
  virtual ~EngineBase() {}
  virtual zc_status set_state(const int *ix, const int *iy, const double *x, const double *y, const double *ux,
                              const double *uy, const double *uz, const double *w, const double *E,
                              const double *B) = 0;
  virtual zc_status set_birth(const int *birth) = 0;
  virtual zc_status set_smooth(int n, const double *sa, const double *sb) = 0;
  virtual zc_status forward(int nsteps, double *objective, double *kin) = 0;
  virtual zc_status backward(double *dw, double *dx, double *dy, double *dux, double *duy, double *duz, double *dE,
                             double *dB) = 0;
  virtual zc_status get_state(int *ix, int *iy, int *alive, double *x, double *y, double *ux, double *uy,
                              double *uz, double *E, double *B) = 0;
  float fwd_ms = 0, bwd_ms = 0;
};

template <class R>
struct DevState {
  int *ix = nullptr, *iy = nullptr, *alive = nullptr;
  R *v = nullptr;  // x, y, ux, uy, uz: 5 arrays of np
  State<R> view(int np) const {
    return State<R>{ix, iy, alive, v, v + np, v + 2 * (size_t)np, v + 3 * (size_t)np, v + 4 * (size_t)np};
  }
};

template <class R>
struct Engine : EngineBase {
  int dev, nx, ny, np, K;
  int mw = 0, obj_kind = 0, obj_row = 0, obj_i0 = 0, obj_i1 = 0;
  double dx, dy, dt, q, m_q;
  float dtf = 0, dxf = 0;  // the float step and cell size the window-move test uses
  size_t pl = 0;           // cells per plane
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  R *w = nullptr;
  int *birth = nullptr;    // step at which each particle starts (null: all at 0)
  DevState<R> cur, nxt;
  R *E = nullptr, *B = nullptr, *J = nullptr, *tmp = nullptr;
  std::vector<std::pair<R, R>> passes;  // current filter passes along x
  std::vector<char> shifts;             // window moves of the last forward run, per step
  // checkpoints (state + E + B) every K steps, and the pre-step states of
  // kseg segments (slot k: step k of the kept stretch)
  std::vector<DevState<R>> ck_s;
  std::vector<R *> ck_f;  // 6 planes each
  int nck = 0;            // checkpoints of the last forward run (slots are reused)
  std::vector<DevState<R>> seg_s;
  std::vector<R *> seg_f;
  int kseg = 1;           // segments the forward run keeps (the last ones)
  int keep0 = 0;          // first step kept by the last forward run
  int steps_done = 0;
  bool have_state = false;
  // reverse
  R *lamE = nullptr, *lamB = nullptr, *lamJ = nullptr, *dwv = nullptr;
  int *d_cross = nullptr, *d_ncross = nullptr;  // cell-crossing particles of a reverse step
  DevState<R> lam;
  double *d_scr = nullptr;  // scratch doubles
  std::vector<void *> owned;

  template <class T>
  zc_status alloc(T **p, size_t n) {
    if (cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
      return afail(ZC_ENOMEM, "adjoint engine: device allocation failed");
    owned.push_back(*p);
    return ZC_OK;
  }
  // one block per state: cells and alive flags (3 x np ints), then the 5 real arrays
  size_t state_bytes() const { return 3 * sizeof(int) * (size_t)np + 5 * sizeof(R) * (size_t)np; }
  zc_status alloc_state(DevState<R> &s) {
    char *b = nullptr;
    TRY_(alloc(&b, state_bytes() + 16));
    s.ix = reinterpret_cast<int *>(b);
    s.iy = s.ix + np;
    s.alive = s.iy + np;
    const size_t off = (3 * sizeof(int) * (size_t)np + 15) / 16 * 16;
    s.v = reinterpret_cast<R *>(b + off);
    return ZC_OK;
  }
  size_t state_span() const { return (3 * sizeof(int) * (size_t)np + 15) / 16 * 16 + 5 * sizeof(R) * (size_t)np; }

  Params<R> params(int n, int shift) const {
    Params<R> P;
    P.nx = nx;
    P.ny = ny;
    P.np = np;
    P.tem = (R)(0.5 * dt / m_q);
    P.dt_dx = (R)(dt / dx);
    P.dt_dy = (R)(dt / dy);
    P.q = (R)q;
    P.qnx = (R)(q * dx / dt);
    P.qny = (R)(q * dy / dt);
    P.mw = mw;
    P.shift = shift;
    P.n = n;
    return P;
  }
  Planes<R> planes(R *f) const { return Planes<R>{f, nx, ny, mw}; }

  zc_status init(const zc_adj_desc *d, double dx_, double dy_) {
    dev = d->device;
    nx = d->nx[0];
    ny = d->nx[1];
    np = d->np;
    K = d->checkpoint_every;
    mw = d->moving_window ? 1 : 0;
    obj_kind = d->objective;
    obj_row = d->objective_row;
    obj_i0 = std::max(0, d->objective_cells[0]);
    obj_i1 = d->objective_cells[1] > 0 ? std::min(d->objective_cells[1], d->nx[0]) : d->nx[0];
    dx = dx_;
    dy = dy_;
    dt = d->dt;
    q = d->q;
    m_q = d->m_q;
    dtf = (float)d->dt;
    dxf = (float)d->box[0] / (float)d->nx[0];
    pl = (size_t)(mw ? nx + 3 : nx) * ny;
    ACK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ACK(cudaEventCreate(&e0));
    ACK(cudaEventCreate(&e1));
    TRY_(alloc(&w, np));
    TRY_(alloc_state(cur));
    TRY_(alloc_state(nxt));
    TRY_(alloc_state(lam));
    TRY_(alloc(&E, 3 * pl));
    TRY_(alloc(&B, 3 * pl));
    TRY_(alloc(&J, 3 * pl));
    TRY_(alloc(&tmp, 3 * pl));
    TRY_(alloc(&lamE, 3 * pl));
    TRY_(alloc(&lamB, 3 * pl));
    TRY_(alloc(&lamJ, 3 * pl));
    TRY_(alloc(&dwv, np));
    TRY_(alloc(&d_cross, np));
    TRY_(alloc(&d_ncross, 1));
    TRY_(alloc(&d_scr, 16));
    // the forward run keeps the pre-step states of its last two segments
    // when they take at most 8 GiB (the reverse sweep then recomputes one
    // segment fewer), else of the last one
    const double slot_bytes = (double)state_span() + 6.0 * sizeof(R) * (double)pl;
    kseg = (2.0 * K * slot_bytes <= 8.0 * (1 << 30)) ? 2 : 1;
    seg_s.resize((size_t)kseg * K);
    seg_f.resize((size_t)kseg * K);
    for (int k = 0; k < kseg * K; ++k) {
      TRY_(alloc_state(seg_s[k]));
      TRY_(alloc(&seg_f[k], 6 * pl));
    }
    return ZC_OK;
  }

  ~Engine() override {
    if (st) cudaStreamSynchronize(st);
    for (void *p : owned) cudaFree(p);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
  }

  zc_status upload(R *dst, const double *src, size_t n) {
    if (!src) return ZC_OK;
    double *t = nullptr;
    ACK(cudaMallocAsync((void **)&t, n * sizeof(double), st));
    ACK(cudaMemcpyAsync(t, src, n * sizeof(double), cudaMemcpyHostToDevice, st));
    k_from_double<R><<<grid_for(n), 256, 0, st>>>(t, dst, n);
    ACK(cudaGetLastError());
    ACK(cudaFreeAsync(t, st));
    return ZC_OK;
  }
  zc_status download(double *dst, const R *src, size_t n) {
    if (!dst) return ZC_OK;
    double *t = nullptr;
    ACK(cudaMallocAsync((void **)&t, n * sizeof(double), st));
    k_to_double<R><<<grid_for(n), 256, 0, st>>>(src, t, n);
    ACK(cudaGetLastError());
    ACK(cudaMemcpyAsync(dst, t, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    ACK(cudaFreeAsync(t, st));
    return ZC_OK;
  }

  zc_status set_state(const int *ix, const int *iy, const double *x, const double *y, const double *ux,
                      const double *uy, const double *uz, const double *wt, const double *Eh,
                      const double *Bh) override {
    ACK(cudaMemcpyAsync(cur.ix, ix, sizeof(int) * np, cudaMemcpyHostToDevice, st));
    ACK(cudaMemcpyAsync(cur.iy, iy, sizeof(int) * np, cudaMemcpyHostToDevice, st));
    std::vector<int> ones(np, 1);
    ACK(cudaMemcpyAsync(cur.alive, ones.data(), sizeof(int) * np, cudaMemcpyHostToDevice, st));
    const State<R> v = cur.view(np);
    TRY_(upload(v.x, x, np));
    TRY_(upload(v.y, y, np));
    TRY_(upload(v.ux, ux, np));
    TRY_(upload(v.uy, uy, np));
    TRY_(upload(v.uz, uz, np));
    TRY_(upload(w, wt, np));
    if (Eh) TRY_(upload(E, Eh, 3 * pl));
    else ACK(cudaMemsetAsync(E, 0, sizeof(R) * 3 * pl, st));
    if (Bh) TRY_(upload(B, Bh, 3 * pl));
    else ACK(cudaMemsetAsync(B, 0, sizeof(R) * 3 * pl, st));
    ACK(cudaStreamSynchronize(st));
    nck = 0;
    steps_done = 0;
    have_state = true;
    return ZC_OK;
  }

  zc_status set_birth(const int *bh) override {
    if (!bh) {
      birth = nullptr;
      return ZC_OK;
    }
    if (!birth) {
      int *b = nullptr;
      TRY_(alloc(&b, np));
      birth = b;
    }
    ACK(cudaMemcpyAsync(birth, bh, sizeof(int) * np, cudaMemcpyHostToDevice, st));
    ACK(cudaStreamSynchronize(st));
    return ZC_OK;
  }

  zc_status set_smooth(int n, const double *sa, const double *sb) override {
    passes.clear();
    for (int k = 0; k < n; ++k) passes.push_back({(R)sa[k], (R)sb[k]});
    return ZC_OK;
  }

  zc_status copy_state(const DevState<R> &dst, const DevState<R> &src) {
    ACK(cudaMemcpyAsync(dst.ix, src.ix, state_span(), cudaMemcpyDeviceToDevice, st));
    return ZC_OK;
  }

  // keeps the pre-step fields of a step in slot k (the particles of a kept
  // step are written there by the step before it)
  zc_status keep_pre_fields(int k) {
    ACK(cudaMemcpyAsync(seg_f[k], E, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(seg_f[k] + 3 * pl, B, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    return ZC_OK;
  }

  // the window moves at step n when (n+1) dt passes the next cell edge
  // (spec_move_window / emf_move_window, particles.c:621, emf.c:650)
  void plan_shifts(int nsteps) {
    shifts.assign(nsteps, 0);
    if (!mw) return;
    int nm = 0;
    for (int n = 0; n < nsteps; ++n) {
      const int it = n + 1;
      if ((it * dtf) > (dxf * (nm + 1))) {
        shifts[n] = 1;
        ++nm;
      }
    }
  }

  // one step of the forward engine: cur -> nxt, E, B advanced
  zc_status step(int n, double *ekin) {
    TRY_(step_into(n, cur, nxt, ekin));
    std::swap(cur, nxt);
    return ZC_OK;
  }

  // one step of the forward engine: particles src -> dst, E, B advanced
  zc_status step_into(int n, const DevState<R> &src, const DevState<R> &dst, double *ekin) {
    const Params<R> P = params(n, shifts[n]);
    ACK(cudaMemsetAsync(J, 0, sizeof(R) * 3 * pl, st));
    k_adj_push<R><<<grid_for(np, 256), 256, 0, st>>>(src.view(np), dst.view(np), w, birth, planes(E), planes(B),
                                                      planes(J), ekin, P);
    ACK(cudaGetLastError());
    // current filter passes along x (current_smooth, em2d/current.c:427-459)
    for (const auto &ps : passes) {
      k_adj_smooth_x<R><<<grid_for(3 * pl), 256, 0, st>>>(J, tmp, nx, ny, mw, ps.first, ps.second);
      std::swap(J, tmp);
    }
    const R hx = (R)(0.5 * dt / dx), hy = (R)(0.5 * dt / dy);
    const R cx = (R)(dt / dx), cy = (R)(dt / dy);
    if (mw) {
      k_adj_yee_b_mw<R><<<grid_for(pl), 256, 0, st>>>(E, B, nx, ny, hx, hy);
      k_adj_yee_e_mw<R><<<grid_for(pl), 256, 0, st>>>(E, B, J, nx, ny, cx, cy, (R)dt);
      k_adj_yee_b_mw<R><<<grid_for(pl), 256, 0, st>>>(E, B, nx, ny, hx, hy);
      if (P.shift) {
        k_adj_shift<R><<<grid_for(3 * pl), 256, 0, st>>>(E, tmp, nx, 3 * pl);
        ACK(cudaMemcpyAsync(E, tmp, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
        k_adj_shift<R><<<grid_for(3 * pl), 256, 0, st>>>(B, tmp, nx, 3 * pl);
        ACK(cudaMemcpyAsync(B, tmp, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
      }
    } else {
      k_adj_yee_b<R><<<grid_for(pl), 256, 0, st>>>(E, B, nx, ny, hx, hy);
      k_adj_yee_e<R><<<grid_for(pl), 256, 0, st>>>(E, B, J, nx, ny, cx, cy, (R)dt);
      k_adj_yee_b<R><<<grid_for(pl), 256, 0, st>>>(E, B, nx, ny, hx, hy);
    }
    ACK(cudaGetLastError());
    return ZC_OK;
  }

  zc_status save_checkpoint(const DevState<R> &from) {
    if (nck == (int)ck_s.size()) {
      DevState<R> s;
      R *f = nullptr;
      TRY_(alloc_state(s));
      TRY_(alloc(&f, 6 * pl));
      ck_s.push_back(s);
      ck_f.push_back(f);
    }
    TRY_(copy_state(ck_s[nck], from));
    ACK(cudaMemcpyAsync(ck_f[nck], E, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(ck_f[nck] + 3 * pl, B, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    ++nck;
    return ZC_OK;
  }

  zc_status restore_checkpoint(int k, const DevState<R> &to) {
    TRY_(copy_state(to, ck_s[k]));
    ACK(cudaMemcpyAsync(E, ck_f[k], sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemcpyAsync(B, ck_f[k] + 3 * pl, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
    return ZC_OK;
  }

  // the objective of the current fields; with seed, the adjoint of its
  // fields goes to lamE / lamB
  R obj_seed() const { return obj_kind == 0 ? (R)(dx * dy) : (R)(2.0 * dx); }
  double obj_scale() const { return obj_kind == 0 ? 0.5 * dx * dy : dx; }
  zc_status objective(double *out, bool seed) {
    ACK(cudaMemsetAsync(d_scr, 0, sizeof(double), st));
    k_adj_objective<R><<<grid_for(6 * pl), 256, 0, st>>>(E, B, seed ? lamE : nullptr, seed ? lamB : nullptr, nx, ny,
                                                          mw, obj_kind, obj_row, obj_i0, obj_i1, obj_seed(), d_scr);
    ACK(cudaGetLastError());
    if (out) {
      double v = 0;
      ACK(cudaMemcpyAsync(&v, d_scr, sizeof(double), cudaMemcpyDeviceToHost, st));
      ACK(cudaStreamSynchronize(st));
      *out = obj_scale() * v;
    }
    return ZC_OK;
  }

  zc_status forward(int nsteps, double *obj, double *kin) override {
    if (!have_state) return afail(ZC_ESTATE, "adjoint engine: no initial state");
    if (nsteps <= 0) return afail(ZC_EINVAL, "adjoint engine: nsteps must be > 0");
    plan_shifts(nsteps);
    ACK(cudaEventRecord(e0, st));
    nck = 0;
    ACK(cudaMemsetAsync(d_scr + 1, 0, sizeof(double), st));
    // the last kseg segments' pre-step states are kept on the way (each
    // kept step writes its particles straight into the next slot): the
    // reverse sweep starts with them and need not recompute those segments
    const int last0 = ((nsteps - 1) / K) * K;
    keep0 = std::max(0, last0 - (kseg - 1) * K);
    for (int n = 0; n < nsteps; ++n) {
      double *ek = n == nsteps - 1 ? d_scr + 1 : nullptr;
      if (n < keep0) {
        if (n % K == 0) TRY_(save_checkpoint(cur));
        TRY_(step(n, ek));
        continue;
      }
      const int k = n - keep0;
      if (k == 0) TRY_(copy_state(seg_s[0], cur));
      if (n % K == 0) TRY_(save_checkpoint(seg_s[k]));
      TRY_(keep_pre_fields(k));
      TRY_(step_into(n, seg_s[k], n + 1 < nsteps ? seg_s[k + 1] : cur, ek));
    }
    steps_done = nsteps;
    ACK(cudaEventRecord(e1, st));
    if (obj) TRY_(objective(obj, false));
    if (kin) {
      // q m_q dx dy sum w utsq/(gamma+1) of the last step (particles.c:1231)
      double v = 0;
      ACK(cudaMemcpyAsync(&v, d_scr + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
      ACK(cudaStreamSynchronize(st));
      *kin = q * m_q * v * dx * dy;
    }
    ACK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&fwd_ms, e0, e1);
    return ZC_OK;
  }

  // reverse of the field part of step n: lamE, lamB after the step in,
  // before the step out; lamJ receives the current's adjoint (before the
  // filter passes)
  zc_status field_reverse(int n) {
    const R hx = (R)(0.5 * dt / dx), hy = (R)(0.5 * dt / dy);
    const R cx = (R)(dt / dx), cy = (R)(dt / dy);
    if (mw) {
      if (shifts[n]) {
        k_adj_shift_T<R><<<grid_for(3 * pl), 256, 0, st>>>(lamE, tmp, nx, 3 * pl);
        ACK(cudaMemcpyAsync(lamE, tmp, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
        k_adj_shift_T<R><<<grid_for(3 * pl), 256, 0, st>>>(lamB, tmp, nx, 3 * pl);
        ACK(cudaMemcpyAsync(lamB, tmp, sizeof(R) * 3 * pl, cudaMemcpyDeviceToDevice, st));
      }
      k_adj_yee_b_T_mw<R><<<grid_for(pl), 256, 0, st>>>(lamB, lamE, nx, ny, hx, hy);
      k_adj_yee_e_T_mw<R><<<grid_for(pl), 256, 0, st>>>(lamE, lamB, lamJ, nx, ny, cx, cy, (R)dt);
      k_adj_yee_b_T_mw<R><<<grid_for(pl), 256, 0, st>>>(lamB, lamE, nx, ny, hx, hy);
    } else {
      k_adj_yee_b_T<R><<<grid_for(pl), 256, 0, st>>>(lamB, lamE, nx, ny, hx, hy);
      k_adj_yee_e_T<R><<<grid_for(pl), 256, 0, st>>>(lamE, lamB, lamJ, nx, ny, cx, cy, (R)dt);
      k_adj_yee_b_T<R><<<grid_for(pl), 256, 0, st>>>(lamB, lamE, nx, ny, hx, hy);
    }
    for (int k = (int)passes.size() - 1; k >= 0; --k) {
      k_adj_smooth_x_T<R><<<grid_for(3 * pl), 256, 0, st>>>(lamJ, tmp, nx, ny, mw, passes[k].first, passes[k].second);
      std::swap(lamJ, tmp);
    }
    ACK(cudaGetLastError());
    return ZC_OK;
  }

  zc_status backward(double *dwh, double *dxh, double *dyh, double *duxh, double *duyh, double *duzh, double *dEh,
                     double *dBh) override {
    if (steps_done <= 0) return afail(ZC_ESTATE, "adjoint engine: run forward first");
    ACK(cudaEventRecord(e0, st));
    // the adjoint of the final fields (the forward run left them in E, B)
    TRY_(objective(nullptr, true));
    ACK(cudaMemsetAsync(lam.v, 0, sizeof(R) * 5 * (size_t)np, st));
    ACK(cudaMemsetAsync(dwv, 0, sizeof(R) * np, st));
    for (int sgi = nck - 1; sgi >= 0; --sgi) {
      const int n0 = sgi * K, n1 = std::min(steps_done, n0 + K);
      // slots of this segment: kept by the forward run, or recomputed from
      // its checkpoint into the first K slots (each step writing its
      // particles straight into the next slot)
      const bool kept = n0 >= keep0;
      const int s0 = kept ? n0 - keep0 : 0;
      if (!kept) {
        TRY_(restore_checkpoint(sgi, seg_s[0]));
        for (int n = n0; n < n1; ++n) {
          TRY_(keep_pre_fields(n - n0));
          if (n + 1 < n1) TRY_(step_into(n, seg_s[n - n0], seg_s[n - n0 + 1], nullptr));
        }
      }
      // walk the segment backwards
      for (int n = n1 - 1; n >= n0; --n) {
        const int k = s0 + n - n0;
        TRY_(field_reverse(n));
        const Params<R> P = params(n, shifts[n]);
        ACK(cudaMemsetAsync(d_ncross, 0, sizeof(int), st));
        k_adj_push_rev<R><<<grid_for(np, 128), 128, 0, st>>>(seg_s[k].view(np), w, birth, planes(seg_f[k]),
                                                              planes(seg_f[k] + 3 * pl), planes(lamJ), lam.view(np),
                                                              lamE, lamB, dwv, d_cross, d_ncross, P);
        k_adj_push_rev_cross<R><<<grid_for(np / 4, 128), 128, 0, st>>>(
            seg_s[k].view(np), w, birth, planes(seg_f[k]), planes(seg_f[k] + 3 * pl), planes(lamJ), lam.view(np),
            lamE, lamB, dwv, d_cross, d_ncross, P);
        ACK(cudaGetLastError());
      }
    }
    ACK(cudaEventRecord(e1, st));
    const State<R> l = lam.view(np);
    TRY_(download(dwh, dwv, np));
    TRY_(download(dxh, l.x, np));
    TRY_(download(dyh, l.y, np));
    TRY_(download(duxh, l.ux, np));
    TRY_(download(duyh, l.uy, np));
    TRY_(download(duzh, l.uz, np));
    TRY_(download(dEh, lamE, 3 * pl));
    TRY_(download(dBh, lamB, 3 * pl));
    // the engine's state goes back to the start of the run
    TRY_(restore_checkpoint(0, cur));
    ACK(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&bwd_ms, e0, e1);
    steps_done = 0;
    return ZC_OK;
  }

  zc_status get_state(int *ix, int *iy, int *alive, double *x, double *y, double *ux, double *uy, double *uz,
                      double *Eh, double *Bh) override {
    if (ix) ACK(cudaMemcpyAsync(ix, cur.ix, sizeof(int) * np, cudaMemcpyDeviceToHost, st));
    if (iy) ACK(cudaMemcpyAsync(iy, cur.iy, sizeof(int) * np, cudaMemcpyDeviceToHost, st));
    if (alive) ACK(cudaMemcpyAsync(alive, cur.alive, sizeof(int) * np, cudaMemcpyDeviceToHost, st));
    const State<R> v = cur.view(np);
    TRY_(download(x, v.x, np));
    TRY_(download(y, v.y, np));
    TRY_(download(ux, v.ux, np));
    TRY_(download(uy, v.uy, np));
    TRY_(download(uz, v.uz, np));
    TRY_(download(Eh, E, 3 * pl));
    TRY_(download(Bh, B, 3 * pl));
    ACK(cudaStreamSynchronize(st));
    return ZC_OK;
  }
};
#undef TRY_

}  // namespace

struct zc_adj {
  int device = 0;
  int nx = 0, ny = 0, np = 0;
  std::unique_ptr<EngineBase> eng;
};

namespace {
struct AdjDevice {
  int prev = -1;
  explicit AdjDevice(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~AdjDevice() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};
}  // namespace

extern "C" {

zc_status zc_adj_create(const zc_adj_desc *d, zc_adj **out) {
  if (!d || !out) return afail(ZC_EINVAL, "null argument");
  *out = nullptr;
  if (d->nx[0] < 2 || d->nx[1] < 2 || d->np < 0 || d->checkpoint_every <= 0)
    return afail(ZC_EINVAL, "adjoint engine: invalid sizes");
  if (!(d->box[0] > 0) || !(d->box[1] > 0) || !(d->dt > 0) || d->m_q == 0)
    return afail(ZC_EINVAL, "adjoint engine: box, dt must be > 0 and m_q non-zero");
  const double dx = d->box[0] / d->nx[0], dy = d->box[1] / d->nx[1];
  const double cour = std::sqrt(1.0 / (1.0 / (dx * dx) + 1.0 / (dy * dy)));
  if (d->dt >= cour) return afail(ZC_EINVAL, "Invalid timestep, courant condition violation");
  if (d->precision != 0 && d->precision != 1) return afail(ZC_EINVAL, "precision must be 0 (float) or 1 (double)");
  if (d->objective != 0 && d->objective != 1) return afail(ZC_EINVAL, "objective must be 0 or 1");
  if (d->objective == 1 && (d->objective_row < 0 || d->objective_row >= d->nx[1]))
    return afail(ZC_EINVAL, "objective row outside the grid");
  AdjDevice g(d->device);
  zc_adj *h = new zc_adj();
  h->device = d->device;
  h->nx = d->nx[0];
  h->ny = d->nx[1];
  h->np = d->np;
  zc_status st;
  if (d->precision == 0) {
    auto *e = new Engine<float>();
    h->eng.reset(e);
    st = e->init(d, dx, dy);
  } else {
    auto *e = new Engine<double>();
    h->eng.reset(e);
    st = e->init(d, dx, dy);
  }
  if (st != ZC_OK) {
    delete h;
    return st;
  }
  *out = h;
  return ZC_OK;
}

zc_status zc_adj_destroy(zc_adj *h) {
  if (!h) return ZC_OK;
  AdjDevice g(h->device);
  delete h;
  return ZC_OK;
}

zc_status zc_adj_set_state(zc_adj *h, const int *ix, const int *iy, const double *x, const double *y,
                           const double *ux, const double *uy, const double *uz, const double *w, const double *E,
                           const double *B) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  if (!ix || !iy || !x || !y || !ux || !uy || !uz || !w) return afail(ZC_EINVAL, "null particle array");
  // every particle inside the grid, with an in-cell position in [0, 1]
  for (int p = 0; p < h->np; ++p)
    if (ix[p] < 0 || ix[p] >= h->nx || iy[p] < 0 || iy[p] >= h->ny || !(x[p] >= 0.0 && x[p] <= 1.0) ||
        !(y[p] >= 0.0 && y[p] <= 1.0))
      return afail(ZC_EINVAL, "adjoint engine: particle outside the grid or its cell");
  AdjDevice g(h->device);
  return h->eng->set_state(ix, iy, x, y, ux, uy, uz, w, E, B);
}

zc_status zc_adj_forward(zc_adj *h, int nsteps, double *objective, double *kinetic) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  AdjDevice g(h->device);
  return h->eng->forward(nsteps, objective, kinetic);
}

zc_status zc_adj_backward(zc_adj *h, double *dw, double *dx, double *dy, double *dux, double *duy, double *duz,
                          double *dE, double *dB) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  AdjDevice g(h->device);
  return h->eng->backward(dw, dx, dy, dux, duy, duz, dE, dB);
}

zc_status zc_adj_get_state(zc_adj *h, int *ix, int *iy, int *alive, double *x, double *y, double *ux, double *uy,
                           double *uz, double *E, double *B) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  AdjDevice g(h->device);
  return h->eng->get_state(ix, iy, alive, x, y, ux, uy, uz, E, B);
}

zc_status zc_adj_set_birth(zc_adj *h, const int *birth) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  AdjDevice g(h->device);
  return h->eng->set_birth(birth);
}

zc_status zc_adj_set_smooth(zc_adj *h, int npasses, const double *sa, const double *sb) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  if (npasses < 0 || (npasses > 0 && (!sa || !sb))) return afail(ZC_EINVAL, "invalid filter passes");
  return h->eng->set_smooth(npasses, sa, sb);
}

zc_status zc_adj_times(zc_adj *h, float *forward_ms, float *backward_ms) {
  if (!h) return afail(ZC_EINVAL, "null handle");
  if (forward_ms) *forward_ms = h->eng->fwd_ms;
  if (backward_ms) *backward_ms = h->eng->bwd_ms;
  return ZC_OK;
}

}  // extern "C"
