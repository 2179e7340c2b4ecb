// zc_api.cu -- host runtime of libzpic_cuda: the C-ABI declared in
// include/zpic_cuda.h.  One zc_sim owns one CUDA stream and all its device
// buffers; nothing here touches global state other than the per-thread
// error message.
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/zpic_cuda.h"
#include "zc_kernels.h"

using namespace zc;

namespace {

thread_local std::string g_err;

zc_status fail(zc_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return s;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(ZC_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

#define TRY(call)                     \
  do {                                \
    zc_status s_ = (call);            \
    if (s_ != ZC_OK) return s_;       \
  } while (0)

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

zc_status load_encoder() {
  if (g_encode) return ZC_OK;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (q != cudaDriverEntryPointSuccess || !fn) return fail(ZC_ECUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return ZC_OK;
}

// 3-D tensor map over `planes` SoA planes of the padded grid
zc_status make_map(CUtensorMap *m, float *base, const Grid &G, int planes, int bw, int bh) {
  cuuint64_t dims[3] = {(cuuint64_t)G.pitch, (cuuint64_t)G.rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)G.pitch * 4, (cuuint64_t)G.plane * 4};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, (cuuint32_t)planes};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ZC_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ZC_OK;
}

template <class T>
zc_status dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(ZC_ENOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T),
                                    cudaGetErrorString(e));
  return ZC_OK;
}

template <class T>
void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

zc_status alloc_particles(Particles &p, long long n) {
  TRY(dalloc(&p.u, n));
  TRY(dalloc(&p.xy, n));
  return ZC_OK;
}

void free_particles(Particles &p) {
  dfree(p.u);
  dfree(p.xy);
}

struct SpeciesState {
  float m_q = -1, q = 0;
  int ppc[2] = {1, 1};
  int iter = 0, n_move = 0;
  // tile layout
  int *d_off = nullptr, *d_cap = nullptr, *d_np = nullptr;  // np: slots in use (particles and holes)
  int *d_vcnt = nullptr;  // particles (not holes) per tile, filled on demand
  std::vector<int> h_off, h_cap;
  long long alloc = 0;   // particles per buffer
  Particles buf[2] = {};
  int cur = 0;
  // spill lists (in: processed this step, out: written this step)
  Particles spill[2] = {};
  int *d_spill_cnt = nullptr;  // [2]
  int spill_cap = 0;
  int max_cap = 0;             // largest tile capacity
  int sort_stage = 0;          // particles a tile's sort stages in shared memory
  int spill_cur = 0;
  // outboxes: leavers posted by one push, pulled by the next (ob[ob_in]
  // holds the pending ones; its counts are all zero when nothing is pending)
  Outbox ob[2] = {};
  long long ob_alloc = 0;
  int ob_in = 0;
  bool pending = false;
  // energy
  double *d_ekin_tile = nullptr, *d_ekin_extra = nullptr, *d_ekin = nullptr;
  // window injection drawn on the device (zc_set_device_injection)
  int dinj = 0;
  zc_column_profile dprof{};
};

// host state that a step changes (buffer parities and counters)
struct Counters {
  int iter = 0, n_move = 0;
  std::vector<int> sp_iter, sp_n_move, cur, spill_cur, ob_in;
  std::vector<bool> pending;
  int eb_cur = 0, j_cur = 0;
  bool j0_zero = false;
  long long launch[ZC_NPHASE] = {};
};

// a captured run of steps, valid from the state it was captured in
struct StepGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int nsteps = 0;
  bool valid = false;
  unsigned long long id = 0;  // unique per capture (batch graphs hold copies)
  Counters before, after;
  // captured with the push launches bracketed by event-record nodes (push-only
  // profiling): the events recorded at capture, and the node pairs, which
  // every replay points at fresh events of the simulation's pool
  bool timed = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> push_ev;
  std::vector<std::pair<cudaGraphNode_t, cudaGraphNode_t>> push_nodes;
};

std::atomic<unsigned long long> g_capture_id{0};

}  // namespace

void zc::set_error_message(const char *msg) { g_err = msg ? msg : ""; }

struct zc_sim {
  int device = 0;
  cudaStream_t st = nullptr;
  int nx = 0, ny = 0;
  float box[2] = {0, 0}, dx[2] = {0, 0}, dt = 0;
  Grid G{};
  float *EB[2] = {nullptr, nullptr};
  int eb_cur = 0;
  float *EBp = nullptr, *extE = nullptr, *extB = nullptr;
  int ext_Et = 0, ext_Bt = 0;
  float3 ext_E0{0, 0, 0}, ext_B0{0, 0, 0};
  float *J[2] = {nullptr, nullptr};
  int j_cur = 0;
  bool j0_zero = false;  // J[0] was cleared by the last Yee launch (no clear needed)
  unsigned long long *Jfix = nullptr;   // deterministic mode: fixed-point J planes
  CUtensorMap tmK_EB[2], tmK_EBp, tmK_J;
  CUtensorMap tmY_EB[2], tmY_J[2];
  int TX = 16, TY = 16, ntx = 0, nty = 0, ntiles = 0;
  std::vector<SpeciesState> sp;
  int xtype = 0, ytype = 0, xlevel = 0, ylevel = 0;
  int mw = 0, n_move = 0, iter = 0;
  int *d_err = nullptr;
  int *h_pinned = nullptr;        // [0] error bits, [2..3] error bits after a block
  double *d_part = nullptr, *d_emf = nullptr;
  int energy_blocks = 0;
  float *stage = nullptr;         // AoS staging for grids
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0;
  zc_inject_fn inj = nullptr;
  void *inj_user = nullptr;
  zc_part *h_inj = nullptr;       // pinned injection staging
  size_t h_inj_cap = 0;
  cudaEvent_t inj_done = nullptr;
  Particles inj_list{};
  long long inj_list_cap = 0;
  int deterministic = 0;
  int fast = 0;                   // FMA build of the push kernels
  int sort_every = 8;             // steps between per-tile cell sorts
  // batches holding this simulation: while it shares the GPU with other
  // runs, its cell sort stages nothing in shared memory (a staged sort block
  // takes most of a multiprocessor's shared memory from the other runs'
  // kernels)
  int batches = 0;
  float slack = 0.5f;
  int accumulated_err = 0;
  int queued_steps = 0;           // steps zc_step_async queued since the last wait
  // per-phase profiling: event pairs recorded during a call, summed on sync
  int profiling = 0;
  // while a timed graph is captured: where the push's event pairs go
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> *cap_ev = nullptr;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  size_t ev_used = 0;
  double prof_ms[ZC_NPHASE] = {};
  long long prof_launch[ZC_NPHASE] = {};
  // replay of captured steps (CUDA graphs): a whole block, and a shorter
  // prefix of a block for the remainder of a call
  int use_graph = 0;
  StepGraph blk, tail;
  // moving-window blocks (every species injecting on the device), one per
  // signature of the block's host decisions (window moves, injected lattice)
  std::vector<StepGraph> mw_blk;
  std::vector<std::vector<long long>> mw_sig;
  int n_relayout = 0, n_capture = 0;
  cudaEvent_t ev_blk[2] = {nullptr, nullptr};
  // per-step energy history on the device: row = 6 field components, then
  // the kinetic energy of every species
  double *d_hist = nullptr;
  bool hist_host = false;         // d_hist is the device address of the caller's host rows
  int *d_hist_n = nullptr;
  int hist_cap = 0, hist_cols = 0, hist_blocks = 0;
  double **d_ekin_ptrs = nullptr;
  KinSum *d_kin_sums = nullptr;   // with a history: the kinetic sums its row kernel makes
  double *d_hist_part = nullptr;
};

namespace {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

cudaEvent_t pool_event(zc_sim *s);

// Brackets a phase with events when profiling is on; counts its launches
// always.
struct Phase {
  zc_sim *s;
  int ph;
  cudaEvent_t b = nullptr;
  bool node = false;  // recorded as a node of the graph being captured
  Phase(zc_sim *s_, int ph_, int nlaunch) : s(s_), ph(ph_) {
    s->prof_launch[ph] += nlaunch;
    if (s->cap_ev && ph == ZC_PHASE_PUSH) {
      if (cudaEventCreate(&b) != cudaSuccess) {
        b = nullptr;
        return;
      }
      node = true;
      cudaEventRecordWithFlags(b, s->st, cudaEventRecordExternal);
      return;
    }
    if (!s->profiling || (s->profiling == 2 && ph != ZC_PHASE_PUSH)) return;
    b = next_event();
    cudaEventRecord(b, s->st);
  }
  ~Phase() {
    if (!b) return;
    if (node) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) {
        cudaEventDestroy(b);
        return;
      }
      cudaEventRecordWithFlags(e, s->st, cudaEventRecordExternal);
      s->cap_ev->push_back({b, e});
      return;
    }
    cudaEvent_t e = next_event();
    cudaEventRecord(e, s->st);
    s->ev_pending.push_back({ph, {b, e}});
  }
  cudaEvent_t next_event() { return pool_event(s); }
};

// the next event of the simulation's pool (reused after collect_profile)
cudaEvent_t pool_event(zc_sim *s) {
  if (s->ev_used == s->ev_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    s->ev_pool.push_back(e);
  }
  return s->ev_pool[s->ev_used++];
}

// sums the recorded phase times (stream must be synchronised)
void collect_profile(zc_sim *s) {
  for (auto &p : s->ev_pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) s->prof_ms[p.first] += ms;
  }
  s->ev_pending.clear();
  s->ev_used = 0;
}

LayoutConst layout(const zc_sim *s) { return LayoutConst{s->TX, s->TY, s->ntx, s->nty, s->nx, s->ny}; }

TileSet tiles(SpeciesState &p, int ntiles) { return TileSet{p.d_off, p.d_cap, p.d_np, ntiles}; }

Spill spill_of(SpeciesState &p, int k) { return Spill{p.spill[k], p.d_spill_cnt + k, p.spill_cap}; }

FixedJ fixed_j(const zc_sim *s) { return FixedJ{s->Jfix, s->G.pitch, s->G.plane, s->J[0]}; }

// outbox slots per tile: room for a moving-window column plus crossers
// (more leavers than slots go to the spill list)
zc_status ensure_outbox(zc_sim *s, SpeciesState &p, int max_cap) {
  // (at most 2^26 slots: the push lists incoming slots in 28-bit fields)
  int per = std::min(1 << 26, std::max(128, ((max_cap / 8) + 31) / 32 * 32));
  long long need = (long long)per * s->ntiles;
  if (per <= p.ob[0].cap && need <= p.ob_alloc) return ZC_OK;
  for (int b = 0; b < 2; ++b) {
    free_particles(p.ob[b].p);
    dfree(p.ob[b].dst);
    TRY(alloc_particles(p.ob[b].p, need));
    TRY(dalloc(&p.ob[b].dst, need));
    if (!p.ob[b].cnt) TRY(dalloc(&p.ob[b].cnt, s->ntiles));
    CK(cudaMemsetAsync(p.ob[b].cnt, 0, sizeof(int) * s->ntiles, s->st));
    p.ob[b].cap = per;
  }
  p.ob_alloc = need;
  p.pending = false;
  return ZC_OK;
}

// moves the particles still waiting in the outboxes into their tiles
zc_status settle(zc_sim *s, SpeciesState &p) {
  if (!p.pending) return ZC_OK;
  Phase ph(s, ZC_PHASE_MIGRATE, 1);
  CK(launch_settle(p.buf[p.cur], tiles(p, s->ntiles), p.ob[p.ob_in], spill_of(p, p.spill_cur), s->d_err, s->ntx,
                   s->nty, s->mw, s->st));
  CK(cudaMemsetAsync(p.ob[p.ob_in].cnt, 0, sizeof(int) * s->ntiles, s->st));
  p.pending = false;
  return ZC_OK;
}

void invalidate_graph(zc_sim *s);

// Tile offsets and capacities from per-tile particle counts: room for the
// count or for the nominal full-density tile, whichever is larger, plus
// slack.  New A/B buffers are allocated when the species' do not hold the
// layout (nbuf then holds them; otherwise nbuf aliases the species').
struct TilePlan {
  std::vector<int> off, cap;
  long long tot = 0;
  bool grow = false;
  Particles nbuf[2] = {};
};

zc_status plan_tiles(zc_sim *s, SpeciesState &p, const std::vector<int> &cnt, TilePlan &pl) {
  const int nt = s->ntiles;
  const long long nominal = (long long)p.ppc[0] * p.ppc[1] * s->TX * s->TY;
  pl.off.assign(nt, 0);
  pl.cap.assign(nt, 0);
  pl.tot = 0;
  int max_cap = 0;
  long long max_fill = 0;
  for (int t = 0; t < nt; ++t) {
    long long base = std::max<long long>(cnt[t], nominal);
    max_fill = std::max(max_fill, base);
    long long c = (long long)std::ceil(base * (1.0 + s->slack)) + 32;
    c = (c + 31) / 32 * 32;
    if (c > (1LL << 30)) return fail(ZC_ENOMEM, "tile capacity too large");
    pl.off[t] = (int)pl.tot;
    pl.cap[t] = (int)c;
    pl.tot += c;
    max_cap = std::max(max_cap, (int)c);
  }
  if (pl.tot >= (1LL << 31)) return fail(ZC_ENOMEM, "species too large for 32-bit tile offsets");
  TRY(ensure_outbox(s, p, max_cap));
  p.max_cap = max_cap;
  // the cell sort stages the fullest tile's particles at this layout plus a
  // quarter (fuller tiles take their excess from global memory): staging
  // room sized to the capacity, three times the particles with a large
  // slack, would leave one sort block a multiprocessor where batched runs
  // share the GPU
  p.sort_stage = (int)std::min<long long>(max_cap, max_fill + max_fill / 4 + 64);
  pl.grow = pl.tot > p.alloc;
  if (pl.grow) {
    TRY(alloc_particles(pl.nbuf[0], pl.tot));
    TRY(alloc_particles(pl.nbuf[1], pl.tot));
  } else {
    pl.nbuf[0] = p.buf[0];
    pl.nbuf[1] = p.buf[1];
  }
  CK(cudaMemcpyAsync(p.d_off, pl.off.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(p.d_cap, pl.cap.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, s->st));
  return ZC_OK;
}

// takes the planned layout as the species' (stream synchronised)
void adopt_tiles(SpeciesState &p, TilePlan &pl) {
  if (pl.grow) {
    free_particles(p.buf[0]);
    free_particles(p.buf[1]);
    p.buf[0] = pl.nbuf[0];
    p.buf[1] = pl.nbuf[1];
    p.alloc = pl.tot;
    p.cur = 0;
  }
  p.h_off = pl.off;
  p.h_cap = pl.cap;
}

// Builds the tile layout of a species from per-tile counts and moves its
// particles (tiles of the current layout, its spill list and an optional
// new list) into it.  Every tile is then sorted by cell (k_cellsort).  The
// order inside a cell is not fixed; the deterministic mode sums currents
// and energies in an order-independent way.
zc_status relayout(zc_sim *s, int k, const Particles *list, int list_n) {
  SpeciesState &p = s->sp[k];
  cudaStream_t st = s->st;
  invalidate_graph(s);
  s->n_relayout += 1;
  TRY(settle(s, p));
  const LayoutConst L = layout(s);
  const int nt = s->ntiles;
  int *d_cnt = nullptr, *d_fill = nullptr, *d_np_old = nullptr, *d_off_old = nullptr;
  TRY(dalloc(&d_cnt, nt));
  TRY(dalloc(&d_fill, nt));
  CK(launch_count_valid(p.buf[p.cur], p.d_off, p.d_np, d_cnt, nt, st));  // holes do not count
  TRY(dalloc(&d_np_old, nt));
  TRY(dalloc(&d_off_old, nt));
  CK(cudaMemcpyAsync(d_np_old, p.d_np, sizeof(int) * nt, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d_off_old, p.d_off, sizeof(int) * nt, cudaMemcpyDeviceToDevice, st));
  int *d_list_n = nullptr;
  TRY(dalloc(&d_list_n, 1));
  CK(cudaMemcpyAsync(d_list_n, &list_n, sizeof(int), cudaMemcpyHostToDevice, st));
  CK(launch_count_list(p.spill[p.spill_cur], p.d_spill_cnt + p.spill_cur, p.spill_cap, d_cnt, L, st));
  if (list && list_n > 0) CK(launch_count_list(*list, d_list_n, list_n, d_cnt, L, st));
  std::vector<int> cnt(nt);
  CK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * nt, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));

  TilePlan pl;
  TRY(plan_tiles(s, p, cnt, pl));
  // destination of the scatter: the buffer that does not hold the particles
  const int src_i = p.cur, tmp_i = 1 - p.cur;
  Particles tmp = pl.grow ? pl.nbuf[1] : p.buf[tmp_i];
  CK(launch_copy_tiles(p.buf[src_i], d_off_old, d_np_old, tmp, p.d_off, d_fill, nt, st));
  CK(launch_scatter_list(p.spill[p.spill_cur], p.d_spill_cnt + p.spill_cur, p.spill_cap, tmp, p.d_off,
                         p.d_cap, d_fill, L, s->d_err, st));
  if (list && list_n > 0)
    CK(launch_scatter_list(*list, d_list_n, list_n, tmp, p.d_off, p.d_cap, d_fill, L, s->d_err, st));
  CK(cudaMemcpyAsync(p.d_np, cnt.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, st));
  // every tile into the other buffer in cell order (the lane-run layout)
  Particles dst = pl.grow ? pl.nbuf[0] : p.buf[src_i];
  CK(launch_cellsort(tmp, dst, p.d_off, p.d_np, L, nt, *std::max_element(cnt.begin(), cnt.end()), s->d_err, st));
  CK(cudaMemsetAsync(p.d_spill_cnt, 0, 2 * sizeof(int), st));
  CK(cudaStreamSynchronize(st));
  adopt_tiles(p, pl);
  dfree(d_cnt);
  dfree(d_fill);
  dfree(d_np_old);
  dfree(d_off_old);
  dfree(d_list_n);
  return ZC_OK;
}

// Loads a list into a species whose tiles and spill list are empty, straight
// into the sorted layout: the per-cell counts of the list (counted while it
// was staged) give the tile counts, the layout, and every cell's first
// position; one scatter then puts every particle where k_cellsort would.
zc_status load_sorted(zc_sim *s, int k, const Particles &list, int n, int *d_cell) {
  SpeciesState &p = s->sp[k];
  cudaStream_t st = s->st;
  invalidate_graph(s);
  s->n_relayout += 1;
  const LayoutConst L = layout(s);
  const int nt = s->ntiles;
  int *d_cnt = nullptr;
  TRY(dalloc(&d_cnt, nt));
  CK(launch_cell_starts(d_cell, d_cnt, L, nt, st));
  std::vector<int> cnt(nt);
  CK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * nt, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  TilePlan pl;
  zc_status r = plan_tiles(s, p, cnt, pl);
  if (r != ZC_OK) {
    dfree(d_cnt);
    return r;
  }
  Particles dst = pl.grow ? pl.nbuf[0] : p.buf[p.cur];
  CK(launch_scatter_sorted(list, n, dst, p.d_off, d_cnt, d_cell, L, st));
  CK(cudaMemcpyAsync(p.d_np, d_cnt, sizeof(int) * nt, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemsetAsync(p.d_spill_cnt, 0, 2 * sizeof(int), st));
  CK(cudaStreamSynchronize(st));
  adopt_tiles(p, pl);
  dfree(d_cnt);
  return ZC_OK;
}

// The device address of a host buffer that the staging kernel may read in
// place: the whole buffer page-locked and mapped (cudaHostAlloc'd or
// registered memory; over the host link the kernel reads it as fast as a
// copy would move it) and 4-byte aligned.  Null for any other buffer, which
// is copied to the device first.
const void *mapped_records(const void *h, size_t bytes) {
  if (!h || bytes == 0 || ((uintptr_t)h & 3)) return nullptr;
  cudaPointerAttributes a0{}, a1{};
  const char *last = (const char *)h + bytes - 1;
  if (cudaPointerGetAttributes(&a0, h) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  if ((const char *)a1.devicePointer - (const char *)a0.devicePointer != (ptrdiff_t)(bytes - 1)) return nullptr;
  return a0.devicePointer;
}

// host AoS -> device SoA list (temporary).  With d_cell, also the particles
// of every cell (nx * ny counters, allocated here, the caller frees them).
zc_status upload_list(zc_sim *s, const zc_part *parts, int n, Particles &list, int **d_cell = nullptr) {
  TRY(alloc_particles(list, std::max(n, 1)));
  int *cell = nullptr;
  if (d_cell) {
    TRY(dalloc(&cell, (size_t)s->nx * s->ny));
    CK(cudaMemsetAsync(cell, 0, sizeof(int) * (size_t)s->nx * s->ny, s->st));
    *d_cell = cell;
  }
  if (n <= 0) return ZC_OK;
  const size_t bytes = sizeof(zc_part) * (size_t)n;
  const void *src = mapped_records(parts, bytes);
  void *d_aos = nullptr;
  if (!src) {
    CK(cudaMalloc(&d_aos, bytes));
    CK(cudaMemcpyAsync(d_aos, parts, bytes, cudaMemcpyHostToDevice, s->st));
    src = d_aos;
  }
  CK(launch_stage_to_list(src, n, list, cell, layout(s), s->d_err, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (d_aos) cudaFree(d_aos);
  return ZC_OK;
}

zc_status check_errors(zc_sim *s, bool relayout_spill) {
  CK(cudaMemcpyAsync(s->h_pinned, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  int e = s->h_pinned[0];
  if (e) {
    CK(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st));
    s->accumulated_err |= e;
  }
  if (relayout_spill && (e & ERR_SPILLED)) {
    // Spilled particles are advanced every step by the spill kernel (global
    // atomics, slower per particle than the tiles); a re-layout (host
    // synchronous, new tile capacities) drains them once enough have piled
    // up to matter, well before the spill list can fill.
    for (size_t k = 0; k < s->sp.size(); ++k) {
      SpeciesState &p = s->sp[k];
      int n = 0;
      CK(cudaMemcpy(&n, p.d_spill_cnt + p.spill_cur, sizeof(int), cudaMemcpyDeviceToHost));
      if (n >= std::max(1024, p.spill_cap / 32)) TRY(relayout(s, (int)k, nullptr, 0));
    }
  }
  if (e & ERR_OVERFLOW) return fail(ZC_EOVERFLOW, "particle spill buffer exhausted: particles were lost");
  if (e & ERR_TIMEOUT) return fail(ZC_ETIMEOUT, "a TMA barrier wait timed out");
  if (e & ERR_ESCAPE) return fail(ZC_EPARTICLE_ESCAPE, "a particle moved more than one cell or left its tile");
  return ZC_OK;
}

// Scale of the push's integer current tile (jsplit).  Every contribution
// is below vmax = 1.5 |q| in magnitude: a segment's Jx is qnx dx' with |dx'|
// <= |mx| = (dt/dx) |ux| / gamma < dt/dx, so |Jx| < |q| (Jy alike), and its Jz
// corner weights times qvz/2 stay below 1.25 |q| (the margin covers the
// fast build's approximate square roots); a warp adds at most 32 of them at
// once.  A tile takes at most n = 3 (largest tile + 8 outboxes)
// contributions per node (three segments per particle).  With 2^cl >= n, L =
// min(22, 31 - cl) keeps the sums of the |m|, |l| <= 2^(L-1) below 2^30; js
// = 2^k with k = 40 (the unit of the deterministic sums) unless n vmax js
// 2^-2L <= 2^30 (the sum of the |h| below 2^31) or 32 vmax js 2^-2L < 2^22
// (the shifter's range) need less.  Deterministic runs require k = 40, so
// that their sums do not depend on the tile layout.
zc_status set_current_scale(zc_sim *s, const SpeciesState &p, PushConst &C) {
  const double vmax = std::max(1.5 * std::fabs((double)p.q), 1e-30);
  const long long n = 3LL * ((long long)p.max_cap + 8LL * p.ob[0].cap) + 1;
  int cl = 0;
  while ((1LL << cl) < n) ++cl;
  if (cl > 28) return fail(ZC_ENOMEM, "tile capacity too large for the integer current tile");
  const int L = std::min(22, 31 - cl);
  const double k1 = std::floor(std::log2(std::ldexp(1.0, 30 + 2 * L) / ((double)n * vmax)));
  const double k2 = std::floor(std::log2(std::ldexp(1.0, 16 + 2 * L) / vmax));
  const int kx = (int)std::max(-60.0, std::min(40.0, std::min(k1, k2)));
  if (s->deterministic && kx < 40)
    return fail(ZC_EINVAL, "charge or tile capacity too large for deterministic (fixed-point) deposition");
  C.js = (float)std::ldexp(1.0, kx);
  C.js_invl = (float)std::ldexp(1.0, -L);
  C.js_twol = (float)std::ldexp(1.0, L);
  C.js_inv2l = (float)std::ldexp(1.0, -2 * L);
  C.js_two2l = (float)std::ldexp(1.0, 2 * L);
  C.js_lo = (float)std::ldexp(1.0, -kx);
  C.js_l = L;
  C.js_det = s->deterministic ? 1LL : 0LL;  // 2^(40 - k), k = 40
  return ZC_OK;
}

zc_status inject_column_device(zc_sim *s, SpeciesState &p);
int column_lattice(const zc_sim *s, const SpeciesState &p, int n_move, ColumnInject &C, unsigned long long &mask);

// kin_later: the step's history row kernel makes the kinetic sum
zc_status spec_advance_impl(zc_sim *s, int k, bool kin_later = false) {
  SpeciesState &p = s->sp[k];
  cudaStream_t st = s->st;
  // moving window: decided after the push, on the species' own counters
  // (spec_move_window, particles.c:621)
  int shift = 0;
  if (s->mw) {
    const int it = p.iter + 1;
    shift = ((it * s->dt) > (s->dx[0] * (p.n_move + 1))) ? 1 : 0;
  }
  PushConst C;
  C.tem = (float)(0.5 * s->dt / p.m_q);
  C.dt_dx = s->dt / s->dx[0];
  C.dt_dy = s->dt / s->dx[1];
  C.qnx = p.q * s->dx[0] / s->dt;
  C.qny = p.q * s->dx[1] / s->dt;
  C.q = p.q;
  C.nx = s->nx;
  C.ny = s->ny;
  C.ntx = s->ntx;
  C.nty = s->nty;
  C.shift = shift;
  C.mw = s->mw;
  TRY(set_current_scale(s, p, C));
  const int in = p.spill_cur, out = 1 - p.spill_cur;
  {
    Phase ph(s, ZC_PHASE_SPILL, 0);
    CK(cudaMemsetAsync(p.d_spill_cnt + out, 0, sizeof(int), st));
    CK(cudaMemsetAsync(p.d_ekin_extra, 0, 2 * sizeof(double), st));
  }
  PushLaunch a;
  a.tm_eb = s->EBp ? &s->tmK_EBp : &s->tmK_EB[s->eb_cur];
  a.pin = p.buf[p.cur];
  a.pout = p.buf[1 - p.cur];
  a.T = tiles(p, s->ntiles);
  a.Oin = p.ob[p.ob_in];
  a.O = p.ob[1 - p.ob_in];
  a.S = spill_of(p, out);
  a.ekin_tile = p.d_ekin_tile;
  a.err = s->d_err;
  a.C = C;
  a.ntiles = s->ntiles;
  a.TX = s->TX;
  a.TY = s->TY;
  a.fast = s->fast;
  a.det = s->deterministic;
  a.fj = fixed_j(s);
  if (s->sort_every > 0 && p.iter % s->sort_every == 0) {
    // keep the tiles sorted by cell (the push warps then share cells)
    Phase ph(s, ZC_PHASE_SORT, 1);
    CK(launch_cellsort(p.buf[p.cur], p.buf[1 - p.cur], p.d_off, p.d_np, layout(s), s->ntiles,
                       s->batches > 0 ? 0 : p.sort_stage, s->d_err, st));
    p.cur = 1 - p.cur;
    a.pin = p.buf[p.cur];
    a.pout = p.buf[1 - p.cur];
  }
  {
    Phase ph(s, ZC_PHASE_PUSH, 1);
    CK(launch_push_tiles(a, st));
  }
  const float *EBpart = s->EBp ? s->EBp : s->EB[s->eb_cur];
  {
    Phase ph(s, ZC_PHASE_SPILL, 1);
    // (normally empty: a grid sized to the run, so that the many small runs
    // of a batch do not launch a full grid each for nothing)
    const int spill_blocks = std::max(1, std::min(152, s->ntiles / 4));
    CK(launch_push_spill(EBpart, s->J[0], fixed_j(s), s->G, p.spill[in], p.d_spill_cnt + in, p.spill_cap,
                         spill_of(p, out), p.d_ekin_extra, s->d_err, C, spill_blocks, s->fast, s->deterministic,
                         st));
  }
  if (s->deterministic) {
    // the float J the rest of the step reads: the fixed-point sum so far
    Phase ph(s, ZC_PHASE_ZERO, 1);
    CK(launch_fixed_to_float(s->Jfix, s->J[0], 3 * s->G.plane, st));
  }
  p.ob_in = 1 - p.ob_in;
  p.pending = true;
  p.cur = 1 - p.cur;
  p.spill_cur = out;
  if (!kin_later) {
    Phase ph(s, ZC_PHASE_KIN_ENERGY, 1);
    CK(launch_sum_energy(p.d_ekin_tile, s->ntiles, p.d_ekin_extra, p.d_ekin, p.q * p.m_q, s->dx[0], s->dx[1],
                         s->deterministic, st));
  }
  p.iter += 1;
  if (shift && p.dinj) {
    p.n_move += 1;
    TRY(inject_column_device(s, p));
  } else if (shift) {
    p.n_move += 1;
    if (!s->inj) return fail(ZC_ESTATE, "moving window needs an injection provider (zc_set_injector)");
    const zc_part *parts = nullptr;
    int n = 0;
    if (s->inj(s->inj_user, k, p.n_move, &parts, &n) != 0)
      return fail(ZC_EINVAL, "injection provider failed");
    if (n > 0) {
      Phase ph(s, ZC_PHASE_WINDOW, 3);
      if ((size_t)n > s->h_inj_cap || n > s->inj_list_cap) {
        CK(cudaStreamSynchronize(st));
        if (s->h_inj) cudaFreeHost(s->h_inj);
        size_t c = (size_t)n * 2 + 1024;
        CK(cudaMallocHost((void **)&s->h_inj, c * sizeof(zc_part)));
        s->h_inj_cap = c;
        free_particles(s->inj_list);
        TRY(alloc_particles(s->inj_list, (long long)c));
        s->inj_list_cap = (long long)c;
      } else {
        CK(cudaEventSynchronize(s->inj_done));  // previous copy out of the pinned buffer is done
      }
      std::memcpy(s->h_inj, parts, sizeof(zc_part) * (size_t)n);
      // pinned AoS -> device list (the list arrays double as the AoS staging)
      void *d_aos = nullptr;
      CK(cudaMallocAsync(&d_aos, sizeof(zc_part) * (size_t)n, st));
      CK(cudaMemcpyAsync(d_aos, s->h_inj, sizeof(zc_part) * (size_t)n, cudaMemcpyHostToDevice, st));
      CK(cudaEventRecord(s->inj_done, st));
      CK(launch_stage_to_list(d_aos, n, s->inj_list, nullptr, layout(s), s->d_err, st));  // no cell counts
      CK(launch_append_list(s->inj_list, n, p.buf[p.cur], tiles(p, s->ntiles), spill_of(p, p.spill_cur),
                            layout(s), s->d_err, st));
      CK(cudaFreeAsync(d_aos, st));
    }
  }
  return ZC_OK;
}

// the column a window move uncovers, drawn on the device for a cold species
// (spec_move_window + spec_inject_particles, em2d/particles.c:476-492,
// 619-640): the ppc lattice of every row of column nx-1 that passes the
// uniform / step / slab test, momenta ufl (a cold species' thermal part is
// zero and so is its per-cell mean).  The lattice offsets and the density
// test use the reference's float and double arithmetic.
// the lattice positions of column nx-1 that pass the density test at window
// offset n_move, in spec_set_x's order (bit q of mask: lattice point q);
// returns their count
int column_lattice(const zc_sim *s, const SpeciesState &p, int n_move, ColumnInject &C, unsigned long long &mask) {
  const zc_column_profile &D = p.dprof;
  C = ColumnInject{};
  mask = 0;
  if (D.type == 1) return 0;  // empty
  C.ix = s->G.nx - 1;
  C.ny = s->G.ny;
  const float dpcx = 1.0f / p.ppc[0], dpcy = 1.0f / p.ppc[1];
  const float start = D.start / s->dx[0] - n_move;
  const float end = D.end / s->dx[0] - n_move;
  int cnt = 0;
  for (int jj = 0; jj < p.ppc[1]; ++jj)
    for (int ii = 0; ii < p.ppc[0]; ++ii) {
      const float x = (float)(dpcx * (ii + 0.5));
      const float y = (float)(dpcy * (jj + 0.5));
      bool take = true;
      if (D.type == 2) take = C.ix + x > start;
      if (D.type == 3) take = C.ix + x > start && C.ix + x < end;
      if (take) {
        mask |= 1ULL << (jj * p.ppc[0] + ii);
        C.px[cnt] = x;
        C.py[cnt] = y;
        ++cnt;
      }
    }
  C.cnt = cnt;
  C.ux = D.ufl[0];
  C.uy = D.ufl[1];
  C.uz = D.ufl[2];
  return cnt;
}

zc_status inject_column_device(zc_sim *s, SpeciesState &p) {
  ColumnInject C;
  unsigned long long mask = 0;
  const int cnt = column_lattice(s, p, p.n_move, C, mask);
  if (cnt == 0) return ZC_OK;
  const int n = C.ny * cnt;
  // sized by zc_set_device_injection for a whole column (no sync here: the
  // step may be under graph capture)
  if (n > s->inj_list_cap) return fail(ZC_ESTATE, "device injection list too small");
  Phase ph(s, ZC_PHASE_WINDOW, 2);
  CK(launch_inject_column(s->inj_list, C, s->st));
  CK(launch_append_list(s->inj_list, n, p.buf[p.cur], tiles(p, s->ntiles), spill_of(p, p.spill_cur), layout(s),
                        s->d_err, s->st));
  return ZC_OK;
}

void smooth_comp(int n, float *sa, float *sb) {  // get_smooth_comp, em2d/current.c:297-304
  float a = -1;
  float b = (4.0 + 2.0 * n) / n;
  float total = 2 * a + b;
  *sa = a / total;
  *sb = b / total;
}

zc_status current_update_impl(zc_sim *s) {
  cudaStream_t st = s->st;
  {
    Phase ph(s, ZC_PHASE_FOLD, s->mw ? 1 : 2);
    CK(launch_fold(s->J[0], s->G, s->mw, st));
  }
  // pass coefficients (current_smooth, em2d/current.c:427-459; the y
  // binomial pass count is xlevel, as at current.c:449)
  SmoothPasses px{}, py{};
  float sa, sb;
  if (s->xtype != 0) {
    for (int i = 0; i < s->xlevel; ++i) px.sa[px.n] = 0.25f, px.sb[px.n++] = 0.5f;
    if (s->xtype == 2) {
      smooth_comp(s->xlevel, &sa, &sb);
      px.sa[px.n] = sa, px.sb[px.n++] = sb;
    }
  }
  if (s->ytype != 0) {
    for (int i = 0; i < s->xlevel; ++i) py.sa[py.n] = 0.25f, py.sb[py.n++] = 0.5f;
    if (s->ytype == 2) {
      smooth_comp(s->ylevel, &sa, &sb);
      py.sa[py.n] = sa, py.sb[py.n++] = sb;
    }
  }
  int c = 0;
  if (px.n > 0 || py.n > 0) {
    Phase ph(s, ZC_PHASE_SMOOTH, 1);
    CK(launch_smooth(s->J[0], s->J[1], s->G, px, py, s->mw, st));
    c = 1;
  }
  s->j_cur = c;
  return ZC_OK;
}

// epart: where the Yee kernel leaves the new fields' energy partials (or null)
zc_status emf_advance_impl(zc_sim *s, double *epart = nullptr) {
  cudaStream_t st = s->st;
  YeeConst Y;
  const float dth = s->dt / 2.0f;
  Y.cxb = dth / s->dx[0];
  Y.cyb = dth / s->dx[1];
  Y.cxe = s->dt / s->dx[0];
  Y.cye = s->dt / s->dx[1];
  Y.dt = s->dt;
  Y.mw = s->mw;
  const int o = 1 - s->eb_cur;
  // the Yee kernel writes the guard cells as the guard-cell update leaves
  // them, and clears the raw deposit buffer once the filter has read it
  const bool gc = s->nx >= 3 && s->ny >= 3;
  float *jz = (s->j_cur == 1) ? s->J[0] : nullptr;
  {
    Phase ph(s, ZC_PHASE_YEE, 1);
    CK(launch_yee(&s->tmY_EB[s->eb_cur], &s->tmY_J[s->j_cur], s->EB[o], s->G, Y, s->d_err, epart, jz, gc, st));
  }
  if (jz) s->j0_zero = true;
  s->eb_cur = o;
  if (!gc) {
    Phase ph(s, ZC_PHASE_EMF_GC, 1);
    CK(launch_emf_gc(s->EB[o], s->G, s->mw, st));
  }
  if (s->EBp) {
    Phase ph(s, ZC_PHASE_EXT, 1);
    CK(launch_ext_add(s->EB[o], s->EBp, s->extE, s->extB, s->ext_Et, s->ext_Bt, s->ext_E0, s->ext_B0, s->G, st));
  }
  s->iter += 1;
  if (s->mw && (s->iter * s->dt) > s->dx[0] * (s->n_move + 1)) {  // emf_move_window, emf.c:650
    Phase ph(s, ZC_PHASE_WINDOW, 1);
    CK(launch_window_shift(s->EB[o], s->EB[1 - o], s->G, st));
    s->eb_cur = 1 - o;
    s->n_move += 1;
  }
  return ZC_OK;
}

// in a step (in_step) a J[0] the last Yee launch cleared is not cleared again
zc_status current_zero_impl(zc_sim *s, bool in_step = false) {
  Phase ph(s, ZC_PHASE_ZERO, 0);
  if (!(in_step && s->j0_zero)) CK(cudaMemsetAsync(s->J[0], 0, sizeof(float) * 3 * s->G.plane, s->st));
  s->j0_zero = false;
  if (s->deterministic) CK(cudaMemsetAsync(s->Jfix, 0, sizeof(unsigned long long) * 3 * s->G.plane, s->st));
  s->j_cur = 0;
  return ZC_OK;
}

zc_status iter_impl(zc_sim *s) {
  TRY(current_zero_impl(s, true));
  // with a history, its row kernel makes the kinetic sums, and the Yee
  // kernel sums the new fields' energy (not under a moving window: the
  // window shift follows it)
  const bool hist = s->d_hist != nullptr;
  for (size_t k = 0; k < s->sp.size(); ++k) TRY(spec_advance_impl(s, (int)k, hist));
  TRY(current_update_impl(s));
  const bool fused = hist && !s->mw;
  TRY(emf_advance_impl(s, fused ? s->d_hist_part : nullptr));
  if (hist) {
    Phase ph(s, ZC_PHASE_HISTORY, fused ? 1 : 2);
    CK(launch_energy_history(fused ? nullptr : s->EB[s->eb_cur], s->G, s->d_hist_part,
                             fused ? yee_blocks(s->G) : s->hist_blocks, s->d_hist, s->d_hist_n, s->hist_cap,
                             s->hist_cols, s->d_ekin_ptrs, s->d_kin_sums, (int)s->sp.size(), s->dx[0], s->dx[1],
                             s->st));
  }
  return ZC_OK;
}

void drop_graph(StepGraph &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  for (auto &pe : g.push_ev) {
    cudaEventDestroy(pe.first);
    cudaEventDestroy(pe.second);
  }
  g.push_ev.clear();
  g.push_nodes.clear();
  g.timed = false;
  g.exec = nullptr;
  g.graph = nullptr;
  g.valid = false;
}

void invalidate_graph(zc_sim *s) {
  drop_graph(s->blk);
  drop_graph(s->tail);
  for (auto &g : s->mw_blk) drop_graph(g);
  s->mw_blk.clear();
  s->mw_sig.clear();
}

// steps per captured block: the buffer parities (particle buffers, outboxes,
// spill lists, field buffers) and the periodic cell sort repeat after it
int block_period(const zc_sim *s) { return s->sort_every > 0 ? 2 * s->sort_every : 2; }

Counters save_counters(const zc_sim *s) {
  Counters c;
  c.iter = s->iter;
  c.n_move = s->n_move;
  for (const auto &p : s->sp) {
    c.sp_iter.push_back(p.iter);
    c.sp_n_move.push_back(p.n_move);
    c.cur.push_back(p.cur);
    c.spill_cur.push_back(p.spill_cur);
    c.ob_in.push_back(p.ob_in);
    c.pending.push_back(p.pending);
  }
  c.eb_cur = s->eb_cur;
  c.j_cur = s->j_cur;
  c.j0_zero = s->j0_zero;
  for (int k = 0; k < ZC_NPHASE; ++k) c.launch[k] = s->prof_launch[k];
  return c;
}

// the buffer parities a captured graph starts from
bool same_parities(const Counters &a, const Counters &b) {
  return a.cur == b.cur && a.spill_cur == b.spill_cur && a.ob_in == b.ob_in && a.eb_cur == b.eb_cur &&
         a.j0_zero == b.j0_zero && (a.iter % 2) == (b.iter % 2);
}

// the graph g holds n steps from the current state (block-aligned)
bool graph_ready(const zc_sim *s, const StepGraph &g, int n) {
  return g.valid && g.nsteps == n && g.timed == (s->profiling == 2) && s->iter % block_period(s) == 0 &&
         same_parities(g.before, save_counters(s));
}

// Captures n steps, starting at a block boundary, as a graph.  Capturing
// does not run anything: the host state advanced by the capture is put
// back afterwards.  Without `instantiate` the graph is only recorded (a
// batch copies it into its own graph); ensure_exec instantiates it when the
// simulation replays it itself.
zc_status capture_steps(zc_sim *s, int n, StepGraph &G, bool instantiate = true) {
  drop_graph(G);
  if (s->iter % block_period(s) != 0) return fail(ZC_ESTATE, "graph capture off a block boundary");
  const Counters before = save_counters(s);
  const int prof = s->profiling;
  // push-only profiling: the graph brackets every push with event-record nodes
  const bool timed = prof == 2;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> evs;
  s->profiling = 0;
  if (timed) s->cap_ev = &evs;
  CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
  zc_status st = ZC_OK;
  for (int k = 0; k < n && st == ZC_OK; ++k) st = iter_impl(s);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->st, &g);
  s->cap_ev = nullptr;
  s->profiling = prof;
  auto drop_events = [&] {
    for (auto &pe : evs) {
      cudaEventDestroy(pe.first);
      cudaEventDestroy(pe.second);
    }
  };
  const Counters after = save_counters(s);
  // put the host state back (nothing ran yet)
  s->iter = before.iter;
  s->n_move = before.n_move;
  for (size_t k = 0; k < s->sp.size(); ++k) {
    SpeciesState &p = s->sp[k];
    p.iter = before.sp_iter[k];
    p.n_move = before.sp_n_move[k];
    p.cur = before.cur[k];
    p.spill_cur = before.spill_cur[k];
    p.ob_in = before.ob_in[k];
    p.pending = before.pending[k];
  }
  s->eb_cur = before.eb_cur;
  s->j_cur = before.j_cur;
  s->j0_zero = before.j0_zero;
  for (int k = 0; k < ZC_NPHASE; ++k) s->prof_launch[k] = before.launch[k];
  if (st != ZC_OK) {
    if (g) cudaGraphDestroy(g);
    drop_events();
    return st;
  }
  if (e != cudaSuccess) {
    drop_events();
    return fail(ZC_ECUDA, "stream capture failed: %s", cudaGetErrorString(e));
  }
  cudaGraphExec_t x = nullptr;
  if (instantiate) {
    const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
    if (ei != cudaSuccess) {
      cudaGraphDestroy(g);
      drop_events();
      return fail(ZC_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(ei));
    }
  }
  G.graph = g;
  G.exec = x;
  G.nsteps = n;
  G.timed = timed;
  if (timed) {
    // the event-record nodes the capture made, in push order
    size_t nn = 0;
    CK(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CK(cudaGraphGetNodes(g, nodes.data(), &nn));
    std::vector<std::pair<cudaEvent_t, cudaGraphNode_t>> rec;
    for (cudaGraphNode_t node : nodes) {
      cudaGraphNodeType ty;
      CK(cudaGraphNodeGetType(node, &ty));
      if (ty != cudaGraphNodeTypeEventRecord) continue;
      cudaEvent_t ev = nullptr;
      CK(cudaGraphEventRecordNodeGetEvent(node, &ev));
      rec.push_back({ev, node});
    }
    auto node_of = [&](cudaEvent_t ev) -> cudaGraphNode_t {
      for (const auto &r : rec)
        if (r.first == ev) return r.second;
      return nullptr;
    };
    for (const auto &pe : evs) {
      const cudaGraphNode_t nb = node_of(pe.first), ne = node_of(pe.second);
      if (!nb || !ne) return fail(ZC_ECUDA, "timed graph: an event-record node is missing");
      G.push_nodes.push_back({nb, ne});
    }
  }
  G.push_ev = std::move(evs);
  G.before = before;
  G.after = after;
  G.valid = true;
  G.id = ++g_capture_id;
  s->n_capture += 1;
  return ZC_OK;
}

// instantiates a graph that was only recorded
zc_status ensure_exec(StepGraph &G) {
  if (G.exec) return ZC_OK;
  const cudaError_t e = cudaGraphInstantiate(&G.exec, G.graph, 0);
  if (e != cudaSuccess) {
    G.exec = nullptr;
    return fail(ZC_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
  }
  return ZC_OK;
}

// the host side of running a captured graph
void account_steps(zc_sim *s, const StepGraph &g) {
  const int n = g.nsteps;
  s->iter += n;
  for (size_t k = 0; k < s->sp.size(); ++k) {
    SpeciesState &p = s->sp[k];
    p.iter += n;
    p.pending = g.after.pending[k];
    p.cur = g.after.cur[k];
    p.spill_cur = g.after.spill_cur[k];
    p.ob_in = g.after.ob_in[k];
    p.n_move += g.after.sp_n_move[k] - g.before.sp_n_move[k];
  }
  s->n_move += g.after.n_move - g.before.n_move;
  s->eb_cur = g.after.eb_cur;
  s->j_cur = g.after.j_cur;
  s->j0_zero = g.after.j0_zero;
  for (int k = 0; k < ZC_NPHASE; ++k) s->prof_launch[k] += g.after.launch[k] - g.before.launch[k];
}

// Captured blocks replace eager steps when graphs are on and nothing in the
// step needs the host: no per-phase event timing, and under a moving window
// every species injecting on the device (a provider calls back into the
// host).
bool graph_possible(const zc_sim *s) {
  if (!s->use_graph || s->sp.empty()) return false;
  // every phase timed: eager; the push timed: replayed graphs time it with
  // their event-record nodes (not under a moving window)
  if (s->profiling == 1 || (s->profiling == 2 && s->mw)) return false;
  if (s->mw)
    for (const auto &p : s->sp)
      if (!p.dinj) return false;
  return true;
}

// launches a captured graph; a timed one first points its push event-record
// nodes at fresh events of the pool (the change holds for this launch on,
// earlier launches keep theirs), read with the eager phases' events
zc_status launch_graph(zc_sim *s, StepGraph &g) {
  TRY(ensure_exec(g));
  if (g.timed)
    for (const auto &pn : g.push_nodes) {
      cudaEvent_t b = pool_event(s), e = pool_event(s);
      CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, pn.first, b));
      CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, pn.second, e));
      s->ev_pending.push_back({ZC_PHASE_PUSH, {b, e}});
    }
  CK(cudaGraphLaunch(g.exec, s->st));
  return ZC_OK;
}

// the host decisions of the next n steps of a moving-window run, replayed
// from the counters with the step's own float tests: per species and step
// whether the window moves (spec_move_window, particles.c:621) and then the
// lattice the injection takes, per step whether the fields move
// (emf_move_window, emf.c:650).  A captured block is valid wherever its
// signature repeats.
std::vector<long long> block_signature(const zc_sim *s, int n) {
  std::vector<long long> sig;
  std::vector<int> it(s->sp.size()), nm(s->sp.size());
  for (size_t k = 0; k < s->sp.size(); ++k) {
    it[k] = s->sp[k].iter;
    nm[k] = s->sp[k].n_move;
  }
  int iter = s->iter, nmove = s->n_move;
  for (int step = 0; step < n; ++step) {
    for (size_t k = 0; k < s->sp.size(); ++k) {
      const int i1 = it[k] + 1;
      const int shift = ((i1 * s->dt) > (s->dx[0] * (nm[k] + 1))) ? 1 : 0;
      it[k] = i1;
      sig.push_back(shift);
      if (shift) {
        nm[k] += 1;
        ColumnInject C;
        unsigned long long mask = 0;
        column_lattice(s, s->sp[k], nm[k], C, mask);
        sig.push_back((long long)mask);
      }
    }
    iter += 1;
    const int fshift = ((iter * s->dt) > s->dx[0] * (nmove + 1)) ? 1 : 0;
    nmove += fshift;
    sig.push_back(fshift);
  }
  return sig;
}

// Runs *nsteps by graph replay where it can: eager steps up to a block
// boundary, whole blocks, then the rest as a prefix of a block (its graph is
// kept for the next call that ends the same way).  The error word of each
// block is copied out behind it and read while the next block runs; a spill
// is drained (which re-lays the species out and invalidates the graphs)
// before going on.
zc_status step_graph(zc_sim *s, int *nsteps) {
  const int P = block_period(s);
  while (*nsteps > 0 && s->iter % P != 0) {
    TRY(iter_impl(s));
    --*nsteps;
  }
  int launched = 0;
  while (*nsteps >= P) {
    if (!graph_ready(s, s->blk, P)) TRY(capture_steps(s, P, s->blk));
    TRY(launch_graph(s, s->blk));
    account_steps(s, s->blk);
    *nsteps -= P;
    const int b = launched & 1;
    CK(cudaMemcpyAsync(s->h_pinned + 2 + b, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaEventRecord(s->ev_blk[b], s->st));
    if (launched > 0) {
      CK(cudaEventSynchronize(s->ev_blk[1 - b]));
      if (s->h_pinned[3 - b]) {
        CK(cudaStreamSynchronize(s->st));
        s->h_pinned[2] = s->h_pinned[3] = 0;
        TRY(check_errors(s, true));
      }
    }
    ++launched;
  }
  if (*nsteps > 0) {
    if (!graph_ready(s, s->tail, *nsteps)) TRY(capture_steps(s, *nsteps, s->tail));
    TRY(launch_graph(s, s->tail));
    account_steps(s, s->tail);
    *nsteps = 0;
  }
  return ZC_OK;
}

// step_graph for a moving window with device injection: blocks are keyed by
// their signature (window moves, injected lattice) as well as the buffer
// parities; a few dozen signatures recur along a run.  The rest of a call
// that is shorter than a block runs eagerly.
zc_status step_graph_mw(zc_sim *s, int *nsteps) {
  const int P = block_period(s);
  while (*nsteps > 0 && s->iter % P != 0) {
    TRY(iter_impl(s));
    --*nsteps;
  }
  constexpr size_t kMaxBlocks = 64;
  int launched = 0;
  while (*nsteps >= P) {
    const std::vector<long long> sig = block_signature(s, P);
    const Counters now = save_counters(s);
    StepGraph *g = nullptr;
    for (size_t i = 0; i < s->mw_blk.size(); ++i)
      if (s->mw_blk[i].valid && s->mw_blk[i].nsteps == P && s->mw_sig[i] == sig &&
          same_parities(s->mw_blk[i].before, now)) {
        g = &s->mw_blk[i];
        break;
      }
    if (!g) {
      if (s->mw_blk.size() >= kMaxBlocks) {
        drop_graph(s->mw_blk.front());
        s->mw_blk.erase(s->mw_blk.begin());
        s->mw_sig.erase(s->mw_sig.begin());
      }
      s->mw_blk.emplace_back();
      s->mw_sig.push_back(sig);
      const zc_status st = capture_steps(s, P, s->mw_blk.back());
      if (st != ZC_OK) {
        s->mw_blk.pop_back();
        s->mw_sig.pop_back();
        return st;
      }
      g = &s->mw_blk.back();
    }
    TRY(ensure_exec(*g));
    CK(cudaGraphLaunch(g->exec, s->st));
    account_steps(s, *g);
    *nsteps -= P;
    const int b = launched & 1;
    CK(cudaMemcpyAsync(s->h_pinned + 2 + b, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaEventRecord(s->ev_blk[b], s->st));
    if (launched > 0) {
      CK(cudaEventSynchronize(s->ev_blk[1 - b]));
      if (s->h_pinned[3 - b]) {
        CK(cudaStreamSynchronize(s->st));
        s->h_pinned[2] = s->h_pinned[3] = 0;
        TRY(check_errors(s, true));
      }
    }
    ++launched;
  }
  return ZC_OK;
}

zc_status grid_up(zc_sim *s, const float *host, float *planes) {
  const size_t n = (size_t)(s->nx + 3) * (s->ny + 3) * 3;
  CK(cudaMemcpyAsync(s->stage, host, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
  CK(launch_aos_to_planes(s->stage, planes, s->G, 3, s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status grid_down(zc_sim *s, const float *planes, float *host) {
  const size_t n = (size_t)(s->nx + 3) * (s->ny + 3) * 3;
  CK(launch_planes_to_aos(planes, s->stage, s->G, 3, s->st));
  CK(cudaMemcpyAsync(host, s->stage, n * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status refresh_particle_fields(zc_sim *s) {
  if (!s->EBp) return ZC_OK;
  CK(launch_ext_add(s->EB[s->eb_cur], s->EBp, s->extE, s->extB, s->ext_Et, s->ext_Bt, s->ext_E0, s->ext_B0, s->G,
                    s->st));
  return ZC_OK;
}

zc_status check_species(zc_sim *s, int k) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (k < 0 || k >= (int)s->sp.size()) return fail(ZC_EINVAL, "invalid species index %d", k);
  return ZC_OK;
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

const char *zc_last_error(void) { return g_err.c_str(); }

const char *zc_status_string(zc_status s) {
  switch (s) {
    case ZC_OK: return "ok";
    case ZC_EINVAL: return "invalid argument";
    case ZC_ENOMEM: return "out of memory";
    case ZC_ECUDA: return "CUDA error";
    case ZC_EPARTICLE_ESCAPE: return "particle escaped its cell";
    case ZC_ETIMEOUT: return "device wait timed out";
    case ZC_EOVERFLOW: return "particle overflow";
    case ZC_ESTATE: return "invalid state";
  }
  return "unknown";
}

zc_status zc_post_device_error(zc_sim *s, zc_status which) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  const int bits = which == ZC_EPARTICLE_ESCAPE ? ERR_ESCAPE
                   : which == ZC_ETIMEOUT       ? ERR_TIMEOUT
                   : which == ZC_EOVERFLOW      ? ERR_OVERFLOW
                                                : 0;
  if (!bits) return fail(ZC_EINVAL, "only the statuses the device reports can be posted");
  // between steps: nothing of this simulation is in flight afterwards
  CK(cudaStreamSynchronize(s->st));
  s->h_pinned[0] = bits;
  CK(cudaMemcpyAsync(s->d_err, s->h_pinned, sizeof(int), cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_sim_create(const zc_sim_desc *d, zc_sim **out) {
  if (!d || !out) return fail(ZC_EINVAL, "null argument");
  *out = nullptr;
  if (d->nx[0] < 2 || d->nx[1] < 2) return fail(ZC_EINVAL, "grid must be at least 2 x 2 cells");
  if (!(d->box[0] > 0) || !(d->box[1] > 0) || !(d->dt > 0)) return fail(ZC_EINVAL, "box and dt must be > 0");
  const float dx0 = d->box[0] / d->nx[0], dx1 = d->box[1] / d->nx[1];
  // Courant condition (em2d/simulation.c:105-110)
  const float cour = sqrtf(1.0f / (1.0f / (dx0 * dx0) + 1.0f / (dx1 * dx1)));
  if (d->dt >= cour)
    return fail(ZC_EINVAL, "Invalid timestep, courant condition violation, dtmax = %f", cour);
  int TX = d->tile[0] > 0 ? d->tile[0] : 16, TY = d->tile[1] > 0 ? d->tile[1] : 16;
  if (!tile_supported(TX, TY)) return fail(ZC_EINVAL, "unsupported tile size %d x %d", TX, TY);
  if ((long long)(d->nx[0] + 3) * (d->nx[1] + 3) > (1LL << 30) || d->nx[0] > 65535 || d->nx[1] > 65535)
    return fail(ZC_EINVAL, "grid too large (at most 65535 cells per axis, 2^30 cells)");
  TRY(load_encoder());

  zc_sim *s = new zc_sim();
  s->device = d->device;
  DeviceGuard g(s->device);
  s->nx = d->nx[0];
  s->ny = d->nx[1];
  s->box[0] = d->box[0];
  s->box[1] = d->box[1];
  s->dx[0] = dx0;
  s->dx[1] = dx1;
  s->dt = d->dt;
  s->TX = TX;
  s->TY = TY;
  s->ntx = (s->nx + TX - 1) / TX;
  s->nty = (s->ny + TY - 1) / TY;
  s->ntiles = s->ntx * s->nty;
  s->deterministic = d->deterministic;
  s->fast = d->fast_math ? 1 : 0;
  s->sort_every = d->sort_every > 0 ? d->sort_every : (d->sort_every < 0 ? 0 : 8);
  s->slack = d->tile_slack > 0 ? d->tile_slack : 0.5f;
  Grid &G = s->G;
  G.nx = s->nx;
  G.ny = s->ny;
  G.pitch = ((s->nx + 3 + 4) + 31) / 32 * 32;
  G.rows = s->ny + 3;
  G.plane = (size_t)G.pitch * G.rows;
  zc_status st = ZC_OK;
#define TRYC(call)              \
  do {                          \
    st = (call);                \
    if (st != ZC_OK) goto bad;  \
  } while (0)
  if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
    st = fail(ZC_ECUDA, "cudaStreamCreate failed");
    goto bad;
  }
  for (int b = 0; b < 2; ++b) {
    TRYC(dalloc(&s->EB[b], 6 * G.plane));
    TRYC(dalloc(&s->J[b], 3 * G.plane));
    cudaMemsetAsync(s->EB[b], 0, sizeof(float) * 6 * G.plane, s->st);
    cudaMemsetAsync(s->J[b], 0, sizeof(float) * 3 * G.plane, s->st);
  }
  if (s->deterministic) {
    TRYC(dalloc(&s->Jfix, 3 * G.plane));
    cudaMemsetAsync(s->Jfix, 0, sizeof(unsigned long long) * 3 * G.plane, s->st);
    if ((s->fast ? prepare_push_tiles_fast_det(TX, TY) : prepare_push_tiles_exact_det(TX, TY)) != cudaSuccess) {
      st = fail(ZC_ECUDA, "deterministic push kernels: shared-memory limit not set");
      goto bad;
    }
  }
  TRYC(dalloc(&s->d_err, 1));
  cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st);
  if (cudaMallocHost((void **)&s->h_pinned, 64 * sizeof(int)) != cudaSuccess) {
    st = fail(ZC_ENOMEM, "cudaMallocHost failed");
    goto bad;
  }
  s->energy_blocks = 8 * 152;  // 64 warps a multiprocessor: enough field reads in flight
  TRYC(dalloc(&s->d_part, 6 * s->energy_blocks));
  TRYC(dalloc(&s->d_emf, 6));
  TRYC(dalloc(&s->stage, (size_t)(s->nx + 3) * (s->ny + 3) * 3));
  {
    const int BW = (TX + 6) & ~3, BH = TY + 3;
    for (int b = 0; b < 2; ++b) {
      TRYC(make_map(&s->tmK_EB[b], s->EB[b], G, 6, BW, BH));
      TRYC(make_map(&s->tmY_EB[b], s->EB[b], G, 6, kYeeBW, kYeeBH));
      TRYC(make_map(&s->tmY_J[b], s->J[b], G, 3, kYeeBW, kYeeBH));
    }
    TRYC(make_map(&s->tmK_J, s->J[0], G, 3, BW, BH));
  }
  if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->inj_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_blk[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_blk[1], cudaEventDisableTiming) != cudaSuccess) {
    st = fail(ZC_ECUDA, "cudaEventCreate failed");
    goto bad;
  }
  if (cudaStreamSynchronize(s->st) != cudaSuccess) {
    st = fail(ZC_ECUDA, "initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
    goto bad;
  }
  *out = s;
  return ZC_OK;
bad:
  zc_sim_destroy(s);
  return st;
#undef TRYC
}

zc_status zc_sim_destroy(zc_sim *s) {
  if (!s) return ZC_OK;
  DeviceGuard g(s->device);
  if (s->st) cudaStreamSynchronize(s->st);
  for (auto &p : s->sp) {
    free_particles(p.buf[0]);
    free_particles(p.buf[1]);
    free_particles(p.spill[0]);
    free_particles(p.spill[1]);
    dfree(p.d_off);
    dfree(p.d_cap);
    dfree(p.d_np);
    dfree(p.d_vcnt);
    for (int b = 0; b < 2; ++b) {
      free_particles(p.ob[b].p);
      dfree(p.ob[b].dst);
      dfree(p.ob[b].cnt);
    }
    dfree(p.d_spill_cnt);
    dfree(p.d_ekin_tile);
    dfree(p.d_ekin_extra);
    dfree(p.d_ekin);
  }
  for (int b = 0; b < 2; ++b) {
    dfree(s->EB[b]);
    dfree(s->J[b]);
  }
  dfree(s->Jfix);
  dfree(s->EBp);
  dfree(s->extE);
  dfree(s->extB);
  free_particles(s->inj_list);
  dfree(s->d_err);
  dfree(s->d_part);
  dfree(s->d_emf);
  dfree(s->stage);
  if (s->h_pinned) cudaFreeHost(s->h_pinned);
  if (s->h_inj) cudaFreeHost(s->h_inj);
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->inj_done) cudaEventDestroy(s->inj_done);
  for (auto e : s->ev_blk)
    if (e) cudaEventDestroy(e);
  invalidate_graph(s);
  if (s->hist_host) s->d_hist = nullptr;  // the caller's rows
  s->hist_host = false;
  dfree(s->d_hist);
  dfree(s->d_hist_n);
  dfree(s->d_hist_part);
  dfree(s->d_ekin_ptrs);
  dfree(s->d_kin_sums);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
  return ZC_OK;
}

zc_status zc_species_create(zc_sim *s, const zc_species_desc *d, const zc_part *parts, int np, int *id) {
  if (!s || !d) return fail(ZC_EINVAL, "null argument");
  if (np < 0 || (np > 0 && !parts)) return fail(ZC_EINVAL, "invalid particle buffer");
  if (d->m_q == 0.0f) return fail(ZC_EINVAL, "m_q must be non-zero");
  if (s->d_hist) return fail(ZC_ESTATE, "species must be created before the energy history is enabled");
  DeviceGuard g(s->device);
  invalidate_graph(s);
  s->sp.emplace_back();
  const int k = (int)s->sp.size() - 1;
  SpeciesState &p = s->sp[k];
  p.m_q = d->m_q;
  p.q = d->q;
  p.ppc[0] = std::max(1, d->ppc[0]);
  p.ppc[1] = std::max(1, d->ppc[1]);
  p.iter = s->iter;
  p.n_move = s->n_move;
  const int nt = s->ntiles;
  TRY(dalloc(&p.d_off, nt));
  TRY(dalloc(&p.d_cap, nt));
  TRY(dalloc(&p.d_np, nt));
  TRY(dalloc(&p.d_vcnt, nt));
  CK(cudaMemsetAsync(p.d_np, 0, sizeof(int) * nt, s->st));
  CK(cudaMemsetAsync(p.d_off, 0, sizeof(int) * nt, s->st));
  CK(cudaMemsetAsync(p.d_cap, 0, sizeof(int) * nt, s->st));
  TRY(dalloc(&p.d_spill_cnt, 2));
  CK(cudaMemsetAsync(p.d_spill_cnt, 0, 2 * sizeof(int), s->st));
  p.spill_cap = std::max(65536, (int)std::min<long long>((long long)np / 32, 1 << 26));
  TRY(alloc_particles(p.spill[0], p.spill_cap));
  TRY(alloc_particles(p.spill[1], p.spill_cap));
  TRY(dalloc(&p.d_ekin_tile, nt));
  TRY(dalloc(&p.d_ekin_extra, 2));  // deterministic mode: two fixed-point words
  TRY(dalloc(&p.d_ekin, 1));
  CK(cudaMemsetAsync(p.d_ekin, 0, sizeof(double), s->st));
  CK(cudaMemsetAsync(p.d_ekin_extra, 0, 2 * sizeof(double), s->st));
  TRY(zc_species_set_particles(s, k, parts, np));
  if (id) *id = k;
  return ZC_OK;
}

zc_status zc_species_create_device(zc_sim *s, float m_q, const int ppc[2], const zc_density *dens, const float ufl[3],
                                   const float uth[3], unsigned long long seed, int *id) {
  if (!s || !ppc) return fail(ZC_EINVAL, "null argument");
  if (m_q == 0.0f) return fail(ZC_EINVAL, "m_q must be non-zero");
  if (ppc[0] < 1 || ppc[1] < 1 || ppc[0] > 32) return fail(ZC_EINVAL, "ppc must be 1..32 along x and >= 1 along y");
  const int type = dens ? dens->type : 0;
  if (type != 0 && type != 1 && type != 2 && type != 3)
    return fail(ZC_EINVAL, "device loading supports uniform, empty, step and slab densities");
  DeviceGuard g(s->device);
  // charge of one particle (spec_new, particles.c:557,576)
  float n = dens ? dens->n : 1.0f;
  if (n == 0.0f) n = 1.0f;
  zc_species_desc d;
  d.m_q = m_q;
  d.q = copysignf(1.0f, m_q) / (ppc[0] * ppc[1]) * fabsf(n);
  d.ppc[0] = ppc[0];
  d.ppc[1] = ppc[1];
  int k = -1;
  TRY(zc_species_create(s, &d, nullptr, 0, &k));
  if (id) *id = k;
  if (type == 1) return ZC_OK;  // empty
  SpeciesState &p = s->sp[k];
  // lattice points of every column inside the profile, tested as spec_set_x
  // tests them (particles.c:187-224): xp = i + lattice x against start/dx,
  // end/dx (floats)
  const float hx = 1.0f / ppc[0], hy = 1.0f / ppc[1];
  std::vector<float> latx(ppc[0]);
  for (int a = 0; a < ppc[0]; ++a) latx[a] = (float)(hx * (a + 0.5));
  const float lo = (type == 2 || type == 3) ? dens->start / s->dx[0] : 0.0f;
  const float hi = (type == 3) ? dens->end / s->dx[0] : 0.0f;
  std::vector<int> colpts(s->nx);
  std::vector<unsigned> colmask(s->nx);
  for (int i = 0; i < s->nx; ++i) {
    unsigned m = 0;
    for (int a = 0; a < ppc[0]; ++a) {
      const float xp = i + latx[a];
      const bool in = (type == 0) || (xp > lo && (type != 3 || xp < hi));
      if (in) m |= 1u << a;
    }
    colmask[i] = m;
    colpts[i] = __builtin_popcount(m);
  }
  const LayoutConst L = layout(s);
  std::vector<int> cnt(s->ntiles);
  for (int t = 0; t < s->ntiles; ++t) {
    const int tx = t % s->ntx, ty = t / s->ntx;
    const int cx0 = tx * s->TX, cy0 = ty * s->TY;
    const int wx = std::min(s->TX, s->nx - cx0), wy = std::min(s->TY, s->ny - cy0);
    long long c = 0;
    for (int li = 0; li < wx; ++li) c += colpts[cx0 + li];
    c *= (long long)ppc[1] * wy;
    if (c > p.h_cap[t]) return fail(ZC_ESTATE, "device loading: tile capacity below the lattice count");
    cnt[t] = (int)c;
  }
  int *d_colpts = nullptr;
  unsigned *d_colmask = nullptr;
  TRY(dalloc(&d_colpts, s->nx));
  TRY(dalloc(&d_colmask, s->nx));
  CK(cudaMemcpyAsync(d_colpts, colpts.data(), sizeof(int) * s->nx, cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(d_colmask, colmask.data(), sizeof(unsigned) * s->nx, cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(p.d_np, cnt.data(), sizeof(int) * s->ntiles, cudaMemcpyHostToDevice, s->st));
  InitConst I;
  I.ppcx = ppc[0];
  I.ppcy = ppc[1];
  I.hx = hx;
  I.hy = hy;
  for (int c = 0; c < 3; ++c) {
    I.uth[c] = uth ? uth[c] : 0.0f;
    I.ufl[c] = ufl ? ufl[c] : 0.0f;
  }
  I.seed_lo = (unsigned)seed;
  I.seed_hi = (unsigned)(seed >> 32);
  CK(launch_init_tiles(p.buf[p.cur], p.d_off, d_colpts, d_colmask, I, L, s->ntiles, s->st));
  CK(cudaStreamSynchronize(s->st));
  dfree(d_colpts);
  dfree(d_colmask);
  invalidate_graph(s);
  return check_errors(s, false);
}

zc_status zc_species_set_particles(zc_sim *s, int k, const zc_part *parts, int np) {
  TRY(check_species(s, k));
  if (np < 0 || (np > 0 && !parts)) return fail(ZC_EINVAL, "invalid particle buffer");
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  CK(cudaMemsetAsync(p.d_np, 0, sizeof(int) * s->ntiles, s->st));
  CK(cudaMemsetAsync(p.d_spill_cnt, 0, 2 * sizeof(int), s->st));
  for (int b = 0; b < 2; ++b)
    if (p.ob[b].cnt) CK(cudaMemsetAsync(p.ob[b].cnt, 0, sizeof(int) * s->ntiles, s->st));
  p.pending = false;
  Particles list{};
  int *d_cell = nullptr;
  zc_status r = upload_list(s, parts, np, list, &d_cell);
  if (r == ZC_OK) r = load_sorted(s, k, list, np, d_cell);
  dfree(d_cell);
  free_particles(list);
  if (r != ZC_OK) return r;
  return check_errors(s, false);
}

zc_status zc_species_inject(zc_sim *s, int k, const zc_part *parts, int np) {
  TRY(check_species(s, k));
  if (np <= 0) return ZC_OK;
  if (!parts) return fail(ZC_EINVAL, "null particle buffer");
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  TRY(settle(s, p));
  Particles list{};
  TRY(upload_list(s, parts, np, list));
  CK(launch_append_list(list, np, p.buf[p.cur], tiles(p, s->ntiles), spill_of(p, p.spill_cur), layout(s), s->d_err,
                        s->st));
  CK(cudaStreamSynchronize(s->st));
  free_particles(list);
  return check_errors(s, true);
}

zc_status zc_species_count(zc_sim *s, int k, int *np) {
  TRY(check_species(s, k));
  if (!np) return fail(ZC_EINVAL, "null argument");
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  TRY(settle(s, p));
  std::vector<int> c(s->ntiles);
  int sc = 0;
  CK(launch_count_valid(p.buf[p.cur], p.d_off, p.d_np, p.d_vcnt, s->ntiles, s->st));
  CK(cudaMemcpyAsync(c.data(), p.d_vcnt, sizeof(int) * s->ntiles, cudaMemcpyDeviceToHost, s->st));
  CK(cudaMemcpyAsync(&sc, p.d_spill_cnt + p.spill_cur, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  long long tot = std::min(sc, p.spill_cap);
  for (int v : c) tot += v;
  *np = (int)tot;
  return ZC_OK;
}

zc_status zc_species_get_particles(zc_sim *s, int k, zc_part *out, int cap, int *np) {
  TRY(check_species(s, k));
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  TRY(settle(s, p));
  std::vector<int> c(s->ntiles);
  int sc = 0;
  CK(launch_count_valid(p.buf[p.cur], p.d_off, p.d_np, p.d_vcnt, s->ntiles, s->st));
  CK(cudaMemcpyAsync(c.data(), p.d_vcnt, sizeof(int) * s->ntiles, cudaMemcpyDeviceToHost, s->st));
  CK(cudaMemcpyAsync(&sc, p.d_spill_cnt + p.spill_cur, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  sc = std::min(sc, p.spill_cap);
  std::vector<long long> doff(s->ntiles);
  long long tot = 0;
  for (int t = 0; t < s->ntiles; ++t) {
    doff[t] = tot;
    tot += c[t];
  }
  const long long n = tot + sc;
  if (np) *np = (int)n;
  if (!out) return ZC_OK;
  if (cap < n) return fail(ZC_EINVAL, "output buffer holds %d particles, %lld needed", cap, n);
  if (n == 0) return ZC_OK;
  long long *d_doff = nullptr;
  int *d_aos = nullptr;
  TRY(dalloc(&d_doff, s->ntiles));
  TRY(dalloc(&d_aos, 7 * n));
  CK(cudaMemcpyAsync(d_doff, doff.data(), sizeof(long long) * s->ntiles, cudaMemcpyHostToDevice, s->st));
  CK(launch_gather_aos(p.buf[p.cur], p.d_off, p.d_np, d_doff, d_aos, s->ntiles, s->st));
  CK(launch_list_to_aos(p.spill[p.spill_cur], p.d_spill_cnt + p.spill_cur, p.spill_cap, d_aos, tot, s->st));
  CK(cudaMemcpyAsync(out, d_aos, sizeof(zc_part) * (size_t)n, cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  dfree(d_doff);
  dfree(d_aos);
  return ZC_OK;
}

zc_status zc_set_device_injection(zc_sim *s, int k, const zc_column_profile *prof) {
  if (!s || !prof) return fail(ZC_EINVAL, "null argument");
  if (k < 0 || k >= (int)s->sp.size()) return fail(ZC_EINVAL, "invalid species");
  if (prof->type < 0 || prof->type > 3) return fail(ZC_EINVAL, "device injection takes uniform, empty, step or slab");
  SpeciesState &p = s->sp[k];
  if (p.ppc[0] <= 0 || p.ppc[1] <= 0 || p.ppc[0] * p.ppc[1] > 64)
    return fail(ZC_EINVAL, "device injection takes up to 64 particles per cell");
  DeviceGuard g(s->device);
  const long long need = (long long)s->G.ny * p.ppc[0] * p.ppc[1];
  if (need > s->inj_list_cap) {
    CK(cudaStreamSynchronize(s->st));
    free_particles(s->inj_list);
    TRY(alloc_particles(s->inj_list, need));
    s->inj_list_cap = need;
  }
  p.dprof = *prof;
  p.dinj = 1;
  invalidate_graph(s);
  return ZC_OK;
}

zc_status zc_set_injector(zc_sim *s, zc_inject_fn fn, void *user) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  s->inj = fn;
  s->inj_user = user;
  return ZC_OK;
}

zc_status zc_set_smooth(zc_sim *s, int xtype, int xlevel, int ytype, int ylevel) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (xtype < 0 || xtype > 2 || ytype < 0 || ytype > 2) return fail(ZC_EINVAL, "invalid smoothing type");
  // em2d/simulation.c:136-144
  if (xtype != 0 && xlevel <= 0) return fail(ZC_EINVAL, "Invalid smooth level along x direction");
  if (ytype != 0 && ylevel <= 0) return fail(ZC_EINVAL, "Invalid smooth level along y direction");
  // at most 15 passes along x (a warp of the filter keeps a halo column per
  // pass on each side) and kMaxSmoothPasses along y
  if ((xtype != 0 && xlevel > 14) || (ytype != 0 && xlevel > 14))
    return fail(ZC_EINVAL, "smoothing level above 14 is not supported");
  invalidate_graph(s);
  s->xtype = xtype;
  s->xlevel = xlevel;
  s->ytype = ytype;
  s->ylevel = ylevel;
  return ZC_OK;
}

zc_status zc_set_moving_window(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  invalidate_graph(s);
  s->mw = 1;
  return ZC_OK;
}

zc_status zc_add_laser(zc_sim *s, const zc_laser *in) {
  if (!s || !in) return fail(ZC_EINVAL, "null argument");
  zc_laser L = *in;
  // parameter checks, em2d/emf.c:245-270
  if (L.fwhm != 0) {
    if (L.fwhm <= 0) return fail(ZC_EINVAL, "Invalid laser FWHM, must be > 0");
    L.rise = L.fwhm;
    L.fall = L.fwhm;
    L.flat = 0.;
  }
  if (L.rise <= 0) return fail(ZC_EINVAL, "Invalid laser RISE, must be > 0");
  if (L.flat < 0) return fail(ZC_EINVAL, "Invalid laser FLAT, must be >= 0");
  if (L.fall <= 0) return fail(ZC_EINVAL, "Invalid laser FALL, must be > 0");
  if (L.type != 0 && L.type != 1) return ZC_OK;  // unknown pulse kinds add nothing (emf.c:341-343)
  DeviceGuard g(s->device);
  LaserConst c;
  c.type = L.type;
  c.start = L.start;
  c.rise = L.rise;
  c.flat = L.flat;
  c.fall = L.fall;
  c.a0 = L.a0;
  c.omega0 = L.omega0;
  c.polarization = L.polarization;
  c.W0 = L.W0;
  c.focus = L.focus;
  c.axis = L.axis;
  c.dx = s->dx[0];
  c.dy = s->dx[1];
  CK(launch_laser(s->EB[s->eb_cur], s->G, c, s->st));
  CK(launch_emf_gc(s->EB[s->eb_cur], s->G, s->mw, s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_set_ext_fld(zc_sim *s, int Et, const float E0[3], const float *Eg, int Bt, const float B0[3],
                         const float *Bg) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (Et < 0 || Et > 2 || Bt < 0 || Bt > 2) return fail(ZC_EINVAL, "Invalid external field type");
  if ((Et == 1 && !E0) || (Bt == 1 && !B0) || (Et == 2 && !Eg) || (Bt == 2 && !Bg))
    return fail(ZC_EINVAL, "missing external field values");
  DeviceGuard g(s->device);
  invalidate_graph(s);
  s->ext_Et = Et;
  s->ext_Bt = Bt;
  if (E0) s->ext_E0 = make_float3(E0[0], E0[1], E0[2]);
  if (B0) s->ext_B0 = make_float3(B0[0], B0[1], B0[2]);
  if (Et == 2) {
    if (!s->extE) TRY(dalloc(&s->extE, 3 * s->G.plane));
    TRY(grid_up(s, Eg, s->extE));
  }
  if (Bt == 2) {
    if (!s->extB) TRY(dalloc(&s->extB, 3 * s->G.plane));
    TRY(grid_up(s, Bg, s->extB));
  }
  if (Et == 0 && Bt == 0) {
    dfree(s->EBp);
    return ZC_OK;
  }
  if (!s->EBp) {
    TRY(dalloc(&s->EBp, 6 * s->G.plane));
    CK(cudaMemsetAsync(s->EBp, 0, sizeof(float) * 6 * s->G.plane, s->st));
    const int BW = (s->TX + 6) & ~3, BH = s->TY + 3;
    TRY(make_map(&s->tmK_EBp, s->EBp, s->G, 6, BW, BH));
  }
  TRY(refresh_particle_fields(s));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_step(zc_sim *s, int nsteps) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (nsteps < 0) return fail(ZC_EINVAL, "nsteps must be >= 0");
  DeviceGuard g(s->device);
  CK(cudaEventRecord(s->ev0, s->st));
  if (graph_possible(s)) TRY(s->mw ? step_graph_mw(s, &nsteps) : step_graph(s, &nsteps));
  for (int n = 0; n < nsteps; ++n) {
    TRY(iter_impl(s));
    // spill lists are drained into the tiles at least every 16 steps
    if ((n & 15) == 15 && n + 1 < nsteps) {
      CK(cudaMemcpyAsync(s->h_pinned, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
      CK(cudaStreamSynchronize(s->st));
      collect_profile(s);
      if (s->h_pinned[0] & ERR_SPILLED) TRY(check_errors(s, true));
    }
  }
  CK(cudaEventRecord(s->ev1, s->st));
  CK(cudaEventSynchronize(s->ev1));
  cudaEventElapsedTime(&s->last_ms, s->ev0, s->ev1);
  collect_profile(s);
  return check_errors(s, true);
}

zc_status zc_step_async(zc_sim *s, int nsteps) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (nsteps < 0) return fail(ZC_EINVAL, "nsteps must be >= 0");
  DeviceGuard g(s->device);
  if (graph_possible(s)) TRY(s->mw ? step_graph_mw(s, &nsteps) : step_graph(s, &nsteps));
  for (int n = 0; n < nsteps; ++n) {
    TRY(iter_impl(s));
    // every 16 queued steps: wait, and drain a spill list that has filled
    if (++s->queued_steps >= 16) {
      CK(cudaMemcpyAsync(s->h_pinned, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
      CK(cudaStreamSynchronize(s->st));
      s->queued_steps = 0;
      collect_profile(s);
      if (s->h_pinned[0]) TRY(check_errors(s, true));
    }
  }
  return ZC_OK;
}

zc_status zc_current_zero(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  TRY(current_zero_impl(s));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_spec_advance(zc_sim *s, int k) {
  TRY(check_species(s, k));
  DeviceGuard g(s->device);
  CK(cudaEventRecord(s->ev0, s->st));
  TRY(spec_advance_impl(s, k));
  CK(cudaEventRecord(s->ev1, s->st));
  CK(cudaEventSynchronize(s->ev1));
  cudaEventElapsedTime(&s->last_ms, s->ev0, s->ev1);
  collect_profile(s);
  return check_errors(s, true);
}

zc_status zc_current_update(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  TRY(current_update_impl(s));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_emf_advance(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  TRY(emf_advance_impl(s));
  CK(cudaStreamSynchronize(s->st));
  return check_errors(s, false);
}

zc_status zc_set_fields(zc_sim *s, const float *E, const float *B) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  if (E) TRY(grid_up(s, E, s->EB[s->eb_cur]));
  if (B) TRY(grid_up(s, B, s->EB[s->eb_cur] + 3 * s->G.plane));
  TRY(refresh_particle_fields(s));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_get_fields(zc_sim *s, float *E, float *B) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  if (E) TRY(grid_down(s, s->EB[s->eb_cur], E));
  if (B) TRY(grid_down(s, s->EB[s->eb_cur] + 3 * s->G.plane, B));
  return ZC_OK;
}

zc_status zc_get_particle_fields(zc_sim *s, float *E, float *B) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  const float *src = s->EBp ? s->EBp : s->EB[s->eb_cur];
  if (E) TRY(grid_down(s, src, E));
  if (B) TRY(grid_down(s, src + 3 * s->G.plane, B));
  return ZC_OK;
}

zc_status zc_get_current(zc_sim *s, float *J) {
  if (!s || !J) return fail(ZC_EINVAL, "null argument");
  DeviceGuard g(s->device);
  return grid_down(s, s->J[s->j_cur], J);
}

struct zc_fence {
  cudaEvent_t ev = nullptr;
};

zc_status zc_copy_grid_async(zc_sim *s, int grid, int comp, float *dst, zc_fence **fence) {
  if (!s || !dst || !fence) return fail(ZC_EINVAL, "null argument");
  *fence = nullptr;
  if (comp < 0 || comp > 2) return fail(ZC_EINVAL, "grid component must be 0, 1 or 2");
  DeviceGuard g(s->device);
  const float *eb = s->EB[s->eb_cur], *ebp = s->EBp ? s->EBp : s->EB[s->eb_cur];
  const float *base = nullptr;
  switch (grid) {
    case ZC_GRID_E: base = eb; break;
    case ZC_GRID_B: base = eb + 3 * s->G.plane; break;
    case ZC_GRID_EPART: base = ebp; break;
    case ZC_GRID_BPART: base = ebp + 3 * s->G.plane; break;
    case ZC_GRID_J: base = s->J[s->j_cur]; break;
    default: return fail(ZC_EINVAL, "unknown grid %d", grid);
  }
  // interior cell (0, 0) sits at buffer column 1 of buffer row 1
  const float *src = base + comp * s->G.plane + s->G.pitch + 1;
  CK(cudaMemcpy2DAsync(dst, sizeof(float) * s->G.nx, src, sizeof(float) * s->G.pitch, sizeof(float) * s->G.nx,
                       s->G.ny, cudaMemcpyDeviceToHost, s->st));
  zc_fence *f = new (std::nothrow) zc_fence;
  if (!f) return fail(ZC_ENOMEM, "fence allocation failed");
  cudaError_t e = cudaEventCreateWithFlags(&f->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(f->ev, s->st);
  if (e != cudaSuccess) {
    if (f->ev) cudaEventDestroy(f->ev);
    delete f;
    return fail(ZC_ECUDA, "fence: %s", cudaGetErrorString(e));
  }
  *fence = f;
  return ZC_OK;
}

zc_status zc_fence_wait(zc_fence *f) {
  if (!f) return fail(ZC_EINVAL, "null fence");
  const cudaError_t e = cudaEventSynchronize(f->ev);
  if (e != cudaSuccess) return fail(ZC_ECUDA, "fence wait: %s", cudaGetErrorString(e));
  return ZC_OK;
}

void zc_fence_destroy(zc_fence *f) {
  if (!f) return;
  if (f->ev) cudaEventDestroy(f->ev);
  delete f;
}

zc_status zc_host_alloc(size_t bytes, void **p) {
  if (!p) return fail(ZC_EINVAL, "null argument");
  *p = nullptr;
  const cudaError_t e = cudaHostAlloc(p, bytes ? bytes : 1, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(ZC_ENOMEM, "pinned host allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
  }
  return ZC_OK;
}

void zc_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

zc_status zc_set_current(zc_sim *s, const float *J) {
  if (!s || !J) return fail(ZC_EINVAL, "null argument");
  DeviceGuard g(s->device);
  TRY(grid_up(s, J, s->J[0]));
  s->j_cur = 0;
  s->j0_zero = false;
  if (s->deterministic) {
    CK(launch_float_to_fixed(s->J[0], s->Jfix, 3 * s->G.plane, s->st));
    CK(cudaStreamSynchronize(s->st));
  }
  return ZC_OK;
}

// queues the field-energy reduction and the copies of the energies to the
// host: written by the reduction kernel itself into page-locked host arrays
// (no copy operations), else through device words and copies
zc_status queue_energy(zc_sim *s, double *emf, double *kin) {
  const int nsp = (int)s->sp.size();
  void *emf_d = emf ? const_cast<void *>(mapped_records(emf, 6 * sizeof(double))) : nullptr;
  void *kin_d = (kin && nsp) ? const_cast<void *>(mapped_records(kin, nsp * sizeof(double))) : nullptr;
  const bool direct = (!emf || (emf_d && ((uintptr_t)emf_d & 7) == 0)) &&
                      (!kin || !nsp || (kin_d && ((uintptr_t)kin_d & 7) == 0)) && nsp <= kEkinRefs && (emf || kin);
  if (direct) {
    EkinRefs K{};
    for (int k = 0; k < nsp; ++k) K.p[k] = s->sp[k].d_ekin;
    CK(launch_energy_direct(s->EB[s->eb_cur], s->G, s->d_part, s->energy_blocks, s->dx[0], s->dx[1], K,
                            kin ? nsp : 0, (double *)emf_d, (double *)kin_d, s->st));
    return ZC_OK;
  }
  if (emf) {
    CK(launch_emf_energy(s->EB[s->eb_cur], s->G, s->d_part, s->energy_blocks, s->d_emf, s->dx[0], s->dx[1], s->st));
    CK(cudaMemcpyAsync(emf, s->d_emf, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  }
  if (kin)
    for (size_t k = 0; k < s->sp.size(); ++k)
      CK(cudaMemcpyAsync(kin + k, s->sp[k].d_ekin, sizeof(double), cudaMemcpyDeviceToHost, s->st));
  return ZC_OK;
}

zc_status zc_energy(zc_sim *s, double emf[6], double *kin) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  TRY(queue_energy(s, emf, kin));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_energy_async(zc_sim *s, double emf[6], double *kin) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  return queue_energy(s, emf, kin);
}

zc_status zc_species_charge(zc_sim *s, int k, float *charge) {
  TRY(check_species(s, k));
  if (!charge) return fail(ZC_EINVAL, "null argument");
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  TRY(settle(s, p));
  const size_t n = (size_t)(s->nx + 1) * (s->ny + 1);
  float *d = nullptr;
  TRY(dalloc(&d, n));
  CK(cudaMemcpyAsync(d, charge, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
  CK(launch_charge(p.buf[p.cur], p.d_off, p.d_np, s->ntiles, p.spill[p.spill_cur], p.d_spill_cnt + p.spill_cur,
                   p.spill_cap, d, s->nx, s->ny, p.q, s->mw, s->st));
  CK(cudaMemcpyAsync(charge, d, n * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  dfree(d);
  return ZC_OK;
}

zc_status zc_species_phasespace(zc_sim *s, int k, int quant1, int quant2, const int pha_nx[2],
                                const float pha_range[4], float *buf) {
  TRY(check_species(s, k));
  if (!pha_nx || !pha_range || !buf) return fail(ZC_EINVAL, "null argument");
  auto valid_q = [](int q) { return q == 1 || q == 2 || q == 4 || q == 5 || q == 6; };
  if (!valid_q(quant1) || !valid_q(quant2)) return fail(ZC_EINVAL, "invalid phase-space quantity");
  if (pha_nx[0] <= 0 || pha_nx[1] <= 0 || !(pha_range[1] != pha_range[0]) || !(pha_range[3] != pha_range[2]))
    return fail(ZC_EINVAL, "invalid phase-space grid");
  DeviceGuard g(s->device);
  SpeciesState &p = s->sp[k];
  TRY(settle(s, p));
  PhaConst P;
  P.q1 = quant1;
  P.q2 = quant2;
  P.n1 = pha_nx[0];
  P.n2 = pha_nx[1];
  P.x1min = pha_range[0];
  P.x2min = pha_range[2];
  P.rdx1 = pha_nx[0] / (pha_range[1] - pha_range[0]);
  P.rdx2 = pha_nx[1] / (pha_range[3] - pha_range[2]);
  P.dx = s->dx[0];
  P.dy = s->dx[1];
  P.q = p.q;
  const size_t n = (size_t)pha_nx[0] * pha_nx[1];
  float *d = nullptr;
  TRY(dalloc(&d, n));
  CK(cudaMemcpyAsync(d, buf, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
  CK(launch_phasespace(p.buf[p.cur], p.d_off, p.d_np, s->ntiles, p.spill[p.spill_cur], p.d_spill_cnt + p.spill_cur,
                       p.spill_cap, d, P, s->st));
  CK(cudaMemcpyAsync(buf, d, n * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  dfree(d);
  return ZC_OK;
}

zc_status zc_get_info(zc_sim *s, zc_info *info) {
  if (!s || !info) return fail(ZC_EINVAL, "null argument");
  info->iter = s->iter;
  info->n_move = s->n_move;
  info->moving_window = s->mw;
  info->n_species = (int)s->sp.size();
  info->nx[0] = s->nx;
  info->nx[1] = s->ny;
  info->tile[0] = s->TX;
  info->tile[1] = s->TY;
  info->ntiles[0] = s->ntx;
  info->ntiles[1] = s->nty;
  info->relayouts = s->n_relayout;
  info->captures = s->n_capture;
  return ZC_OK;
}

zc_status zc_grid_view_get(zc_sim *s, zc_grid_view *v) {
  if (!s || !v) return fail(ZC_EINVAL, "null argument");
  v->E = s->EB[s->eb_cur];
  v->B = s->EB[s->eb_cur] + 3 * s->G.plane;
  v->J = s->J[s->j_cur];
  v->plane = s->G.plane;
  v->pitch = s->G.pitch;
  v->rows = s->G.rows;
  v->stream = (void *)s->st;
  return ZC_OK;
}

zc_status zc_synchronize(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  s->queued_steps = 0;
  collect_profile(s);
  return check_errors(s, true);
}

zc_status zc_set_profiling(zc_sim *s, int mode) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (mode < 0 || mode > 2) return fail(ZC_EINVAL, "profiling mode must be 0, 1 or 2");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  collect_profile(s);
  s->profiling = mode;
  return ZC_OK;
}

zc_status zc_get_profile(zc_sim *s, double ms[ZC_NPHASE], long long launches[ZC_NPHASE]) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  collect_profile(s);
  for (int k = 0; k < ZC_NPHASE; ++k) {
    if (ms) ms[k] = s->prof_ms[k];
    if (launches) launches[k] = s->prof_launch[k];
  }
  return ZC_OK;
}

zc_status zc_reset_profile(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  collect_profile(s);
  for (int k = 0; k < ZC_NPHASE; ++k) {
    s->prof_ms[k] = 0;
    s->prof_launch[k] = 0;
  }
  return ZC_OK;
}

const char *zc_phase_name(int p) {
  static const char *names[ZC_NPHASE] = {"push", "spill", "migrate", "kin_energy", "zero",  "fold",   "smooth",
                                         "yee",  "emf_gc", "ext",   "window",     "sort", "history"};
  return (p >= 0 && p < ZC_NPHASE) ? names[p] : "unknown";
}

zc_status zc_last_step_ms(zc_sim *s, float *ms) {
  if (!s || !ms) return fail(ZC_EINVAL, "null argument");
  *ms = s->last_ms;
  return ZC_OK;
}

zc_status zc_set_graphs(zc_sim *s, int on) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  if (!on) invalidate_graph(s);
  s->use_graph = on ? 1 : 0;
  return ZC_OK;
}

zc_status history_setup(zc_sim *s, double *rows, int max_steps);

zc_status zc_history_enable(zc_sim *s, int max_steps) { return history_setup(s, nullptr, max_steps); }

zc_status zc_history_stream(zc_sim *s, double *rows, int max_steps) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (max_steps > 0 && !rows) return fail(ZC_EINVAL, "null row buffer");
  return history_setup(s, rows, max_steps);
}

zc_status history_setup(zc_sim *s, double *rows, int max_steps) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (max_steps < 0) return fail(ZC_EINVAL, "max_steps must be >= 0");
  if (s->sp.size() + 6 > 64) return fail(ZC_EINVAL, "energy history holds at most 58 species");
  DeviceGuard g(s->device);
  CK(cudaStreamSynchronize(s->st));
  invalidate_graph(s);
  if (s->hist_host) s->d_hist = nullptr;  // the caller's rows
  s->hist_host = false;
  dfree(s->d_hist);
  dfree(s->d_hist_n);
  dfree(s->d_hist_part);
  dfree(s->d_ekin_ptrs);
  dfree(s->d_kin_sums);
  s->hist_cap = 0;
  s->hist_cols = 0;
  if (max_steps == 0) return ZC_OK;
  const int cols = 6 + (int)s->sp.size();
  // a small grid gets few blocks (each thread sums >= 4 cells), so that a
  // per-step history stays cheap
  const long long cells = (long long)s->nx * s->ny;
  s->hist_blocks = (int)std::max<long long>(1, std::min<long long>(s->energy_blocks, (cells + 1023) / 1024));
  if (rows) {
    // the caller's page-locked rows, written by the device step by step
    void *d = const_cast<void *>(mapped_records(rows, sizeof(double) * (size_t)max_steps * cols));
    if (!d || ((uintptr_t)d & 7))
      return fail(ZC_EINVAL, "history rows must be page-locked host memory (cudaHostAlloc), 8-byte aligned");
    s->d_hist = static_cast<double *>(d);
    s->hist_host = true;
  } else {
    TRY(dalloc(&s->d_hist, (size_t)max_steps * cols));
  }
  TRY(dalloc(&s->d_hist_n, 1));
  // partials of the standalone energy pass or of the Yee kernel
  TRY(dalloc(&s->d_hist_part, 6 * (size_t)std::max(s->hist_blocks, yee_blocks(s->G))));
  TRY(dalloc(&s->d_ekin_ptrs, std::max<size_t>(1, s->sp.size())));
  TRY(dalloc(&s->d_kin_sums, std::max<size_t>(1, s->sp.size())));
  std::vector<double *> ptrs;
  std::vector<KinSum> sums;
  for (auto &p : s->sp) {
    ptrs.push_back(p.d_ekin);
    sums.push_back(KinSum{p.d_ekin_tile, p.d_ekin_extra, s->ntiles, s->deterministic, p.q * p.m_q});
  }
  if (!ptrs.empty()) {
    CK(cudaMemcpyAsync(s->d_ekin_ptrs, ptrs.data(), sizeof(double *) * ptrs.size(), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->d_kin_sums, sums.data(), sizeof(KinSum) * sums.size(), cudaMemcpyHostToDevice, s->st));
  }
  CK(cudaMemsetAsync(s->d_hist_n, 0, sizeof(int), s->st));
  CK(cudaStreamSynchronize(s->st));
  s->hist_cap = max_steps;
  s->hist_cols = cols;
  return ZC_OK;
}

zc_status zc_history_get(zc_sim *s, double *out, int cap_rows, int *nrows, int *ncols) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  DeviceGuard g(s->device);
  int n = 0;
  if (s->d_hist) {
    CK(cudaMemcpyAsync(&n, s->d_hist_n, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
  }
  if (nrows) *nrows = n;
  if (ncols) *ncols = s->hist_cols;
  if (!out || n == 0) return ZC_OK;
  if (cap_rows < n) return fail(ZC_EINVAL, "output buffer holds %d rows, %d recorded", cap_rows, n);
  CK(cudaMemcpyAsync(out, s->d_hist, sizeof(double) * (size_t)n * s->hist_cols,
                     s->hist_host ? cudaMemcpyDefault : cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

zc_status zc_history_reset(zc_sim *s) {
  if (!s) return fail(ZC_EINVAL, "null simulation handle");
  if (!s->d_hist) return ZC_OK;
  DeviceGuard g(s->device);
  CK(cudaMemsetAsync(s->d_hist_n, 0, sizeof(int), s->st));
  CK(cudaStreamSynchronize(s->st));
  return ZC_OK;
}

}  // extern "C"

// ===========================================================================
// batched runs
// ===========================================================================
struct zc_batch {
  std::vector<zc_sim *> sims;
  int device = 0;
  int period = 0;
  cudaStream_t st = nullptr;  // start and end of a call, its timing
  // one graph per run length (a whole block, a prefix for the remainder):
  // every member of a group's captured steps as a parallel branch
  struct Parent {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int nsteps = 0;
    bool valid = false;
    std::vector<unsigned long long> ids;  // the member captures it copies
    std::vector<cudaGraphNode_t> nodes;   // their child nodes
  };
  // the members are dealt into groups of about equal particle capacity,
  // each with its own stream and graphs: a group starts as soon as its own
  // graph is recorded (the first block of the next group is recorded while
  // it runs), and the groups do not wait for one another between blocks
  struct Group {
    std::vector<int> members;  // member indices, heaviest first
    int off = 0;               // its first slot in the error-word arrays
    cudaStream_t st = nullptr;
    Parent blk, tail;
    cudaEvent_t ev_blk[2] = {nullptr, nullptr};
    cudaEvent_t ev_end = nullptr;
  };
  std::vector<Group> groups;
  std::vector<int> group_of;  // member index -> group
  int **d_errp = nullptr;     // every member's error word, in group order
  int *d_errs = nullptr;      // their copy after a block, [2][n]
  int *h_errs = nullptr;      // pinned, [2][n]
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> ev_sim;  // one per member, joins of its stream
  float last_ms = 0;
  bool marked = false;  // the members count this batch (zc_sim::batches)
};

namespace {

void drop_parent(zc_batch::Parent &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g = zc_batch::Parent{};
}

void drop_groups(zc_batch *b) {
  for (auto &G : b->groups) {
    if (G.st) cudaStreamSynchronize(G.st);
    drop_parent(G.blk);
    drop_parent(G.tail);
    for (auto e : {G.ev_blk[0], G.ev_blk[1], G.ev_end})
      if (e) cudaEventDestroy(e);
    if (G.st) cudaStreamDestroy(G.st);
  }
  b->groups.clear();
}

// the group count a batch of n members takes by default: one group up to
// 32 members, then one more per 32 up to 8
int default_groups(int n) { return std::max(1, std::min(8, n / 32)); }

// deals the members into `ng` groups: heaviest first (most particle
// capacity), in snake order, so that the groups carry about the same work
// and every group's branches start with its longest chains
zc_status form_groups(zc_batch *b, int ng) {
  const int n = (int)b->sims.size();
  ng = std::max(1, std::min(ng, n));
  drop_groups(b);
  std::vector<int> order(n);
  std::vector<long long> weight(n, 0);
  for (int k = 0; k < n; ++k) {
    order[k] = k;
    for (const auto &p : b->sims[k]->sp) weight[k] += p.alloc;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return weight[a] > weight[c]; });
  b->groups.resize(ng);
  b->group_of.assign(n, 0);
  for (int j = 0; j < n; ++j) {
    const int r = j / ng, q = j % ng;
    const int g = (r % 2 == 0) ? q : ng - 1 - q;
    b->groups[g].members.push_back(order[j]);
    b->group_of[order[j]] = g;
  }
  std::vector<int *> ptrs;
  for (auto &G : b->groups) {
    G.off = (int)ptrs.size();
    for (int k : G.members) ptrs.push_back(b->sims[k]->d_err);
    if (cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking) != cudaSuccess)
      return fail(ZC_ECUDA, "cudaStreamCreate failed");
    for (auto *e : {&G.ev_blk[0], &G.ev_blk[1], &G.ev_end})
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess)
        return fail(ZC_ECUDA, "cudaEventCreate failed");
  }
  CK(cudaMemcpy(b->d_errp, ptrs.data(), sizeof(int *) * n, cudaMemcpyHostToDevice));
  return ZC_OK;
}

// makes `pg` run n steps of every member of group G from its current
// state, recapturing what is stale
zc_status batch_ready(zc_batch *b, zc_batch::Group &G, zc_batch::Parent &pg, int n) {
  const std::vector<int> &mem = G.members;
  const bool have = pg.valid && pg.nsteps == n && pg.ids.size() == mem.size();
  bool ok = have;
  // the members to (re)capture, recorded by a few host threads at once
  // (each member captures on its own stream; nothing runs)
  std::vector<int> todo;
  for (int k : mem) {
    zc_sim *s = b->sims[k];
    if (!graph_ready(s, (n == b->period) ? s->blk : s->tail, n)) todo.push_back(k);
  }
  if (!todo.empty()) {
    const int nt = (int)std::min<size_t>(todo.size(), std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
    std::vector<zc_status> res(nt, ZC_OK);
    std::vector<std::string> msg(nt);
    auto work = [&](int w) {
      if (cudaSetDevice(b->device) != cudaSuccess) {
        res[w] = ZC_ECUDA;
        msg[w] = "cudaSetDevice failed in a capture thread";
        return;
      }
      for (size_t i = w; i < todo.size() && res[w] == ZC_OK; i += nt) {
        zc_sim *s = b->sims[todo[i]];
        res[w] = capture_steps(s, n, (n == b->period) ? s->blk : s->tail, false);
        if (res[w] != ZC_OK) msg[w] = g_err;
      }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nt; ++w) pool.emplace_back(work, w);
    work(0);
    for (auto &t : pool) t.join();
    for (int w = 0; w < nt; ++w)
      if (res[w] != ZC_OK) return fail(res[w], "%s", msg[w].c_str());
  }
  for (size_t j = 0; j < mem.size(); ++j) {
    zc_sim *s = b->sims[mem[j]];
    StepGraph &g = (n == b->period) ? s->blk : s->tail;
    if (have && pg.ids[j] != g.id) {
      // a member was captured again (after a re-layout): its copy in the
      // instantiated graph takes the new parameters in place when the
      // topology is unchanged, else everything is rebuilt
      if (cudaGraphExecChildGraphNodeSetParams(pg.exec, pg.nodes[j], g.graph) == cudaSuccess) {
        pg.ids[j] = g.id;
      } else {
        cudaGetLastError();
        ok = false;
      }
    }
  }
  if (ok) return ZC_OK;
  drop_parent(pg);
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  // the members' branches are added heaviest first (the group's order), so
  // that the longest chains start first and the block does not end on them
  pg.nodes.assign(mem.size(), nullptr);
  for (size_t j = 0; j < mem.size(); ++j) {
    StepGraph &sg = (n == b->period) ? b->sims[mem[j]]->blk : b->sims[mem[j]]->tail;
    cudaGraphNode_t node;
    const cudaError_t e = cudaGraphAddChildGraphNode(&node, g, nullptr, 0, sg.graph);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return fail(ZC_ECUDA, "cudaGraphAddChildGraphNode failed: %s", cudaGetErrorString(e));
    }
    pg.nodes[j] = node;
  }
  cudaGraphExec_t x = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ZC_ECUDA, "batch graph instantiation failed: %s", cudaGetErrorString(e));
  }
  pg.graph = g;
  pg.exec = x;
  pg.nsteps = n;
  pg.valid = true;
  pg.ids.clear();
  for (int k : mem) pg.ids.push_back(((n == b->period) ? b->sims[k]->blk : b->sims[k]->tail).id);
  return ZC_OK;
}

}  // namespace

extern "C" {

zc_status zc_batch_create(zc_sim *const *sims, int nsims, zc_batch **out) {
  if (!sims || nsims <= 0 || !out) return fail(ZC_EINVAL, "invalid batch members");
  *out = nullptr;
  const int dev = sims[0] ? sims[0]->device : 0;
  int period = 0;
  for (int k = 0; k < nsims; ++k) {
    zc_sim *s = sims[k];
    if (!s) return fail(ZC_EINVAL, "null member %d", k);
    if (s->device != dev) return fail(ZC_EINVAL, "members must share one device");
    if (s->mw) return fail(ZC_EINVAL, "member %d has a moving window", k);
    if (s->sp.empty()) return fail(ZC_EINVAL, "member %d has no species", k);
    if (k == 0) period = block_period(s);
    if (block_period(s) != period) return fail(ZC_EINVAL, "members must share sort_every");
    for (int j = 0; j < k; ++j)
      if (sims[j] == s) return fail(ZC_EINVAL, "member %d appears twice", k);
  }
  DeviceGuard g(dev);
  zc_batch *b = new zc_batch();
  b->sims.assign(sims, sims + nsims);
  b->device = dev;
  b->period = period;
  zc_status st = ZC_OK;
  auto bad = [&](zc_status r) {
    zc_batch_destroy(b);
    return r;
  };
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess)
    return bad(fail(ZC_ECUDA, "cudaStreamCreate failed"));
  if ((st = dalloc(&b->d_errp, nsims)) != ZC_OK) return bad(st);
  if ((st = dalloc(&b->d_errs, 2 * (size_t)nsims)) != ZC_OK) return bad(st);
  if (cudaMallocHost((void **)&b->h_errs, 2 * sizeof(int) * nsims) != cudaSuccess)
    return bad(fail(ZC_ENOMEM, "cudaMallocHost failed"));
  std::memset(b->h_errs, 0, 2 * sizeof(int) * nsims);
  if (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
    return bad(fail(ZC_ECUDA, "cudaEventCreate failed"));
  b->ev_sim.assign(nsims, nullptr);
  for (auto &e : b->ev_sim)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return bad(fail(ZC_ECUDA, "cudaEventCreate failed"));
  if ((st = form_groups(b, default_groups(nsims))) != ZC_OK) return bad(st);
  for (zc_sim *s : b->sims) {
    s->batches += 1;
    invalidate_graph(s);  // recorded blocks hold the sort of a run alone
  }
  b->marked = true;
  *out = b;
  return ZC_OK;
}

zc_status zc_batch_set_groups(zc_batch *b, int ngroups) {
  if (!b) return fail(ZC_EINVAL, "null batch handle");
  DeviceGuard g(b->device);
  const int n = (int)b->sims.size();
  return form_groups(b, ngroups > 0 ? std::min(ngroups, n) : default_groups(n));
}

zc_status zc_batch_get_groups(zc_batch *b, int *ngroups) {
  if (!b || !ngroups) return fail(ZC_EINVAL, "null argument");
  *ngroups = (int)b->groups.size();
  return ZC_OK;
}

zc_status zc_batch_destroy(zc_batch *b) {
  if (!b) return ZC_OK;
  DeviceGuard g(b->device);
  if (b->st) cudaStreamSynchronize(b->st);
  drop_groups(b);
  if (b->marked)
    for (zc_sim *s : b->sims) {
      s->batches -= 1;
      if (s->batches == 0) invalidate_graph(s);  // recorded blocks hold the batch's sort
    }
  dfree(b->d_errp);
  dfree(b->d_errs);
  if (b->h_errs) cudaFreeHost(b->h_errs);
  for (auto e : {b->ev0, b->ev1})
    if (e) cudaEventDestroy(e);
  for (auto e : b->ev_sim)
    if (e) cudaEventDestroy(e);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return ZC_OK;
}

zc_status zc_batch_step(zc_batch *b, int nsteps) {
  if (!b) return fail(ZC_EINVAL, "null batch handle");
  if (nsteps < 0) return fail(ZC_EINVAL, "nsteps must be >= 0");
  DeviceGuard g(b->device);
  const int n = (int)b->sims.size();
  const int P = b->period;
  for (zc_sim *s : b->sims) {
    if (s->mw) return fail(ZC_ESTATE, "a member has a moving window");
    if (block_period(s) != P) return fail(ZC_ESTATE, "a member changed its sort_every");
    if (s->profiling) return fail(ZC_ESTATE, "a member has profiling on");
  }
  CK(cudaEventRecord(b->ev0, b->st));
  for (zc_sim *s : b->sims) {
    CK(cudaEventRecord(s->ev0, b->st));
    CK(cudaStreamWaitEvent(s->st, s->ev0, 0));
  }
  // members off a block boundary step eagerly on their own streams up to
  // it; the whole blocks every member can then take, and a common prefix of
  // a block for the rest, run as batch graphs; what is left, eagerly
  std::vector<int> lead(n);
  int blocks = nsteps / P;
  bool aligned = true;
  for (int k = 0; k < n; ++k) {
    zc_sim *s = b->sims[k];
    lead[k] = std::min(nsteps, (P - s->iter % P) % P);
    for (int i = 0; i < lead[k]; ++i) TRY(iter_impl(s));
    blocks = std::min(blocks, (nsteps - lead[k]) / P);
    aligned = aligned && lead[k] == 0;
  }
  const int rest = aligned ? nsteps - blocks * P : 0;
  if (blocks > 0 || rest > 0) {
    for (int k = 0; k < n; ++k) {
      CK(cudaEventRecord(b->ev_sim[k], b->sims[k]->st));
      CK(cudaStreamWaitEvent(b->groups[b->group_of[k]].st, b->ev_sim[k], 0));
    }
    for (int i = 0; i < blocks; ++i) {
      const int slot = i & 1;
      for (auto &G : b->groups) {
        const int m = (int)G.members.size();
        TRY(batch_ready(b, G, G.blk, P));
        CK(cudaGraphLaunch(G.blk.exec, G.st));
        for (int k : G.members) account_steps(b->sims[k], b->sims[k]->blk);
        int *dst = b->d_errs + (size_t)slot * n + G.off;
        CK(launch_gather_words(b->d_errp + G.off, m, dst, G.st));
        CK(cudaMemcpyAsync(b->h_errs + (size_t)slot * n + G.off, dst, sizeof(int) * m, cudaMemcpyDeviceToHost,
                           G.st));
        CK(cudaEventRecord(G.ev_blk[slot], G.st));
      }
      if (i > 0) {
        // the previous block's error words, read while this block runs
        for (auto &G : b->groups) CK(cudaEventSynchronize(G.ev_blk[1 - slot]));
        bool any = false;
        for (int k = 0; k < n; ++k) any |= b->h_errs[(size_t)(1 - slot) * n + k] != 0;
        if (any) {
          for (auto &G : b->groups) CK(cudaStreamSynchronize(G.st));
          std::memset(b->h_errs, 0, 2 * sizeof(int) * n);
          for (int k = 0; k < n; ++k) {
            zc_sim *s = b->sims[k];
            TRY(check_errors(s, true));  // a spill re-lays a member out
            CK(cudaEventRecord(b->ev_sim[k], s->st));
            CK(cudaStreamWaitEvent(b->groups[b->group_of[k]].st, b->ev_sim[k], 0));
          }
        }
      }
    }
    if (rest > 0) {
      for (auto &G : b->groups) {
        TRY(batch_ready(b, G, G.tail, rest));
        CK(cudaGraphLaunch(G.tail.exec, G.st));
        for (int k : G.members) account_steps(b->sims[k], b->sims[k]->tail);
      }
    }
    for (auto &G : b->groups) {
      CK(cudaEventRecord(G.ev_end, G.st));
      for (int k : G.members) CK(cudaStreamWaitEvent(b->sims[k]->st, G.ev_end, 0));
    }
  }
  for (int k = 0; k < n; ++k) {
    zc_sim *s = b->sims[k];
    const int m = nsteps - lead[k] - blocks * P - rest;
    for (int i = 0; i < m; ++i) TRY(iter_impl(s));
  }
  for (zc_sim *s : b->sims) {
    CK(cudaEventRecord(s->ev1, s->st));
    CK(cudaStreamWaitEvent(b->st, s->ev1, 0));
  }
  CK(cudaEventRecord(b->ev1, b->st));
  CK(cudaEventSynchronize(b->ev1));
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  for (zc_sim *s : b->sims) TRY(check_errors(s, true));
  return ZC_OK;
}

zc_status zc_batch_last_ms(zc_batch *b, float *ms) {
  if (!b || !ms) return fail(ZC_EINVAL, "null argument");
  *ms = b->last_ms;
  return ZC_OK;
}

}  // extern "C"
