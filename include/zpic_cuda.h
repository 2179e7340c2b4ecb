/*
 * zpic_cuda.h -- C-ABI of libzpic_cuda, the GB300 (sm_103a) implementation of
 * the ZPIC em2d electromagnetic PIC time step.
 *
 * Plain C types only: pointers, sizes, status codes.  Device state lives
 * behind an opaque zc_sim handle; every handle owns one CUDA stream, so
 * handles are independent of each other (the reference itself is
 * single-threaded and non-reentrant, em2d/random.c:16-17, particles.c:26-27).
 *
 * Host buffers use the reference layouts:
 *   particles  zc_part records, identical to t_part (em2d/particles.h:29-37)
 *   grids      float3 interleaved, (nx+3)*(ny+3) cells with 1 lower and 2
 *              upper guard cells per axis, row stride nx+3, cell (0,0) at
 *              offset 1+(nx+3)  (em2d/emf.c:59-89, em2d/current.c:33-53)
 *
 * Nothing here calls exit(): invalid input returns ZC_EINVAL and the message
 * is kept for zc_last_error(); the reference's exit(-1) behaviour is
 * restored, where wanted, by the drop-in layer above this ABI.
 */
#ifndef ZPIC_CUDA_H
#define ZPIC_CUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ZC_API __attribute__((visibility("default")))
#else
#define ZC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ZC_OK = 0,
    ZC_EINVAL = 1,            /* invalid argument (Courant, smoothing, laser, ...) */
    ZC_ENOMEM = 2,            /* device or host allocation failed */
    ZC_ECUDA = 3,             /* a CUDA runtime call failed */
    ZC_EPARTICLE_ESCAPE = 4,  /* a particle moved more than one cell in a step */
    ZC_ETIMEOUT = 5,          /* a bounded device wait (TMA barrier) gave up */
    ZC_EOVERFLOW = 6,         /* particle overflow buffer exhausted: particles lost */
    ZC_ESTATE = 7             /* call not valid in the current state */
} zc_status;

/* particle record, same layout as t_part (em2d/particles.h:29-37) */
typedef struct {
    int ix, iy;
    float x, y;
    float ux, uy, uz;
} zc_part;

typedef struct zc_sim zc_sim;

typedef struct {
    int nx[2];              /* cells along x, y */
    float box[2];           /* box size, simulation units */
    float dt;               /* time step */
    int device;             /* CUDA device ordinal */
    int tile[2];            /* particle tile size in cells (0,0 -> 16 x 16) */
    int deterministic;      /* 1: fixed-order current deposition, bit-reproducible runs */
    float tile_slack;       /* spare tile capacity, fraction (<=0 -> 0.5) */
    int fast_math;          /* 0: push rounds every float32 operation as the reference C
                               (bit-identical particles); 1: FMA-contracted push */
    int sort_every;         /* steps between per-tile cell sorts (0 -> 8, <0 never) */
} zc_sim_desc;

typedef struct {
    float m_q;              /* mass over charge */
    float q;                /* charge of one simulation particle (spec->q) */
    int ppc[2];             /* particles per cell (for reporting only) */
} zc_species_desc;

/* laser pulse, same fields as t_emf_laser (em2d/emf.h:134-157) */
typedef struct {
    int type;               /* 0 plane, 1 gaussian */
    float start, fwhm, rise, flat, fall;
    float a0, omega0, polarization;
    float W0, focus, axis;
} zc_laser;

typedef struct {
    int iter;               /* completed steps (emf->iter) */
    int n_move;             /* moving-window shifts so far */
    int moving_window;
    int n_species;
    int nx[2];
    int tile[2];
    int ntiles[2];
    int relayouts;          /* tile re-layouts so far (uploads, spills drained) */
    int captures;           /* graph captures so far (zc_set_graphs, batches) */
} zc_info;

/* Device view of the grids for zero-copy consumers (e.g. PyTorch): SoA
 * planes [component][row][column] of `pitch` floats per row, `rows` rows,
 * buffer coordinates (column i+1, row j+1) for cell (i, j). */
typedef struct {
    float *E;               /* 3 planes: Ex, Ey, Ez (B follows E in memory) */
    float *B;               /* 3 planes: Bx, By, Bz */
    float *J;               /* 3 planes: Jx, Jy, Jz */
    size_t plane;           /* floats per plane */
    int pitch, rows;
    void *stream;           /* cudaStream_t of the handle */
} zc_grid_view;

/* Moving-window injection provider: called on the host when the window moves
 * (spec_move_window, em2d/particles.c:619-640) with the species index and the
 * updated n_move; it must return the particles of the new right-most column
 * (cell indices already in the shifted frame).  The buffer stays owned by the
 * caller until the next call. */
typedef int (*zc_inject_fn)(void *user, int species, int n_move, const zc_part **parts, int *np);

/* --- lifetime ---------------------------------------------------------- */
/* replaces emf_new + current_new + the Courant check of sim_new
 * (em2d/simulation.c:93-112, em2d/emf.c:56-115, em2d/current.c:30-79) */
ZC_API zc_status zc_sim_create(const zc_sim_desc *desc, zc_sim **out);
/* replaces sim_delete (em2d/simulation.c:212-222) */
ZC_API zc_status zc_sim_destroy(zc_sim *sim);

/* --- species ------------------------------------------------------------- */
/* registers a species whose initial particles were injected on the host by
 * spec_new (em2d/particles.c:535-612) and uploads them */
ZC_API zc_status zc_species_create(zc_sim *sim, const zc_species_desc *desc, const zc_part *parts,
                            int np, int *species_id);
/* density profile of a species loaded on the device (t_density,
 * em2d/particles.h:60-83): type 0 uniform, 1 empty, 2 step (from start),
 * 3 slab (start..end); n the density */
typedef struct {
    int type;
    float n;
    float start, end;
} zc_density;
/* loads a species on the device (spec_set_x / spec_set_u,
 * em2d/particles.c:85-354): the ppc lattice of every cell inside the profile
 * (the positions spec_new gives), thermal momenta uth * N(0,1) from a
 * counter-based generator (Philox4x32-10 keyed by `seed`), the mean momentum
 * of each cell removed and the drift ufl added; written straight into the
 * tile layout in cell order.  Momenta are statistically, not bitwise, those
 * of the reference's generator.  ppc[0] <= 32. */
ZC_API zc_status zc_species_create_device(zc_sim *sim, float m_q, const int ppc[2], const zc_density *density,
                                          const float ufl[3], const float uth[3], unsigned long long seed,
                                          int *species_id);
/* replaces the device particles of a species (host edits between steps,
 * Species.add / Species.particles writes, python/source/em2d.pyx:238-312) */
ZC_API zc_status zc_species_set_particles(zc_sim *sim, int species, const zc_part *parts, int np);
/* appends particles (moving-window injection, em2d/particles.c:476-492) */
ZC_API zc_status zc_species_inject(zc_sim *sim, int species, const zc_part *parts, int np);
/* copies the particles back in tile order; *np receives the count; `cap`
 * is the room in `out` (records).  out == NULL only queries the count. */
ZC_API zc_status zc_species_get_particles(zc_sim *sim, int species, zc_part *out, int cap, int *np);
ZC_API zc_status zc_species_count(zc_sim *sim, int species, int *np);
ZC_API zc_status zc_set_injector(zc_sim *sim, zc_inject_fn fn, void *user);
/* Window injection drawn on the device for a cold species (uth = 0), instead
 * of the provider: after each window move, the species' ppc lattice in every
 * row of column nx-1 that passes the density test, with momenta ufl
 * (spec_move_window + spec_inject_particles + spec_set_x/spec_set_u,
 * em2d/particles.c:159-354, 476-492, 619-640).  Profiles: 0 uniform,
 * 1 empty, 2 step (start), 3 slab (start, end).  The reference's generator
 * is not advanced (a cold species draws nothing from it that matters, but a
 * later thermal draw would see a different sequence). */
typedef struct {
    int type;
    float start, end;
    float ufl[3];
} zc_column_profile;
ZC_API zc_status zc_set_device_injection(zc_sim *sim, int species, const zc_column_profile *prof);

/* --- configuration ------------------------------------------------------- */
/* replaces sim_set_smooth (em2d/simulation.c:134-147) */
ZC_API zc_status zc_set_smooth(zc_sim *sim, int xtype, int xlevel, int ytype, int ylevel);
/* replaces sim_set_moving_window (em2d/simulation.c:154-163) */
ZC_API zc_status zc_set_moving_window(zc_sim *sim);
/* replaces emf_add_laser (em2d/emf.c:242-350) */
ZC_API zc_status zc_add_laser(zc_sim *sim, const zc_laser *laser);
/* replaces emf_set_ext_fld (em2d/emf.c:764-831).  type 0 none, 1 uniform
 * (value in E0/B0), 2 custom (grid in reference layout, evaluated on the
 * host from the user's callback for every buffer cell). */
ZC_API zc_status zc_set_ext_fld(zc_sim *sim, int E_type, const float E0[3], const float *E_grid,
                         int B_type, const float B0[3], const float *B_grid);

/* --- the step ------------------------------------------------------------ */
/* sim_iter x nsteps (em2d/simulation.c:45-56) */
ZC_API zc_status zc_step(zc_sim *sim, int nsteps);
/* zc_step without the wait at the end: the steps are queued on the
 * simulation's stream and the call returns (it waits only every 16 queued
 * steps, to look at the spill list; with graph replay on, whole blocks are
 * queued as graphs and the wait trails one block behind).  Device errors
 * of queued steps are returned by the next waiting call (zc_synchronize,
 * zc_step, zc_energy, ...).  With zc_energy_async or zc_history_stream a
 * run reports every step without idling the device between steps. */
ZC_API zc_status zc_step_async(zc_sim *sim, int nsteps);
/* the phases of sim_iter, for callers that drive them one by one */
ZC_API zc_status zc_current_zero(zc_sim *sim);                 /* em2d/current.c:98-107 */
ZC_API zc_status zc_spec_advance(zc_sim *sim, int species);    /* em2d/particles.c:1104-1269 */
ZC_API zc_status zc_current_update(zc_sim *sim);               /* em2d/current.c:171-183 */
ZC_API zc_status zc_emf_advance(zc_sim *sim);                  /* em2d/emf.c:688-716 */

/* --- data ---------------------------------------------------------------- */
/* E and B in reference layout; either pointer may be NULL */
ZC_API zc_status zc_set_fields(zc_sim *sim, const float *E_buf, const float *B_buf);
ZC_API zc_status zc_get_fields(zc_sim *sim, float *E_buf, float *B_buf);
/* fields seen by the particles (E_part / B_part, em2d/emf.h:96-97) */
ZC_API zc_status zc_get_particle_fields(zc_sim *sim, float *E_buf, float *B_buf);
ZC_API zc_status zc_get_current(zc_sim *sim, float *J_buf);

/* Diagnostics without a stall: one component (0, 1, 2) of one grid's
 * interior, nx * ny floats with x fastest (the layout of the reference's
 * emf_report / current_report buffers, em2d/emf.c:368-482,
 * em2d/current.c:194-281), copied into host memory after the work already
 * on the handle's stream.  The call returns at once; `*fence` completes
 * when `dst` holds the data (`dst` must stay valid until then, and pinned
 * memory from zc_host_alloc keeps the copy asynchronous). */
enum { ZC_GRID_E = 0, ZC_GRID_B = 1, ZC_GRID_EPART = 2, ZC_GRID_BPART = 3, ZC_GRID_J = 4 };
typedef struct zc_fence zc_fence;
ZC_API zc_status zc_copy_grid_async(zc_sim *sim, int grid, int comp, float *dst, zc_fence **fence);
ZC_API zc_status zc_fence_wait(zc_fence *fence);  /* may be called from any thread */
ZC_API void zc_fence_destroy(zc_fence *fence);
/* page-locked host memory for asynchronous copies */
ZC_API zc_status zc_host_alloc(size_t bytes, void **ptr);
ZC_API void zc_host_free(void *ptr);

/* ------------------------------------------------------------------------- */
/* em1d: the reference's one-dimensional electromagnetic step (em1d/*.c)     */
/* ------------------------------------------------------------------------- */
/* One handle = one 1-D simulation on one GPU: push + zigzag deposit
 * (em1d/particles.c:707-1062), current update with binomial / compensated
 * filtering (em1d/current.c:111-330), Yee advance with periodic, open (Mur)
 * or moving-window boundaries (em1d/emf.c:379-580).  Grids are the
 * reference's float3 buffers of nx + 3 cells (one lower, two upper guard
 * cells); particles the reference's 20-byte record. */
typedef struct zc1_sim zc1_sim;
typedef struct zc1_desc {
    int nx;
    float box;
    float dt;
    int device;
    int open_fields;     /* Mur boundaries (emf.bc_type = EMF_BC_OPEN) */
    int open_particles;  /* particles leaving [0, nx) are removed (PART_BC_OPEN) */
    int moving_window;   /* sim_set_moving_window: fields and current without boundary */
    int sort_every;      /* cell sort interval of the particle buffers (0: 16) */
    int push_ctas;       /* most CTAs of the push and sort kernels (0: one particle per
                            thread up to a full wave; simulations that run side by side
                            do better with fewer, each thread then pushing several) */
} zc1_desc;
typedef struct zc1_part {  /* em1d/particles.h:29-35 */
    int ix;
    float x, ux, uy, uz;
} zc1_part;
typedef struct zc1_species_desc {
    float m_q, q;        /* q: the species' particle charge (spec_new, particles.c:530-545) */
    int ppc;
    float ufl[3], uth[3];
    int density;         /* injection profile: 0 uniform, 1 empty, 2 step, 3 slab */
    float start, end;
} zc1_species_desc;
ZC_API zc_status zc1_create(const zc1_desc *desc, zc1_sim **sim);
ZC_API void zc1_destroy(zc1_sim *sim);
/* particles as loaded by the caller (e.g. the reference's spec_new); a
 * moving window injects cold particles (ufl) into column nx-1 by the profile.
 * Species are added before the first zc1_step. */
ZC_API zc_status zc1_add_species(zc1_sim *sim, const zc1_species_desc *desc, const zc1_part *parts, int np,
                                 int *species);
ZC_API zc_status zc1_set_smooth(zc1_sim *sim, int type, int level);  /* 0 none, 1 binomial, 2 compensated */
ZC_API zc_status zc1_set_fields(zc1_sim *sim, const float *E_buf, const float *B_buf);
ZC_API zc_status zc1_get_fields(zc1_sim *sim, float *E_buf, float *B_buf);
ZC_API zc_status zc1_get_current(zc1_sim *sim, float *J_buf);
/* adds a laser pulse to E and B (emf_add_laser, em1d/emf.c:191-260; the
 * plane-wave fields of zc_laser, whose type, W0, focus and axis are unused).
 * Periodic simulations then copy the guard cells, as the reference does for
 * its default boundary; its decks add the laser before they switch to open or
 * moving-window boundaries, where the copies are zero for a pulse inside the
 * box. */
ZC_API zc_status zc1_add_laser(zc1_sim *sim, const zc_laser *laser);
/* sim_iter x nsteps (em1d/simulation.c:45-56); waits for the steps and
 * reports their errors */
ZC_API zc_status zc1_step(zc1_sim *sim, int nsteps);
/* the same steps, only enqueued on the simulation's stream: independent
 * simulations (a parameter scan) then run side by side on one GPU.  The
 * host still waits when a particle buffer may have to grow.  Errors of the
 * steps surface at zc1_synchronize. */
ZC_API zc_status zc1_step_async(zc1_sim *sim, int nsteps);
/* waits for the enqueued steps; returns their first error */
ZC_API zc_status zc1_synchronize(zc1_sim *sim);
/* device time from the first step enqueued after the previous wait to the
 * last wait (CUDA events on the simulation's stream) */
ZC_API zc_status zc1_last_step_ms(zc1_sim *sim, float *ms);
/* particles pushed so far by a species, summed over its steps (particle-steps) */
ZC_API zc_status zc1_species_pushed(zc1_sim *sim, int species, long long *pushed);
/* kernels the steps of this simulation have launched so far */
ZC_API zc_status zc1_get_launches(zc1_sim *sim, long long *launches);
/* per-kernel device time: with profiling on, every kernel of a step is
 * bracketed by CUDA events (event-record nodes in the step graphs, which are
 * then replayed one at a time; this costs time of its own, so leave it off
 * for timing runs).  zc1_set_profile resets the
 * sums; zc1_get_profile returns milliseconds and launches per kind since then:
 * the push (with boundaries, compaction and injection), the cell sort (three
 * kernels) and the fields kernel (current filter and field advance). */
enum { ZC1_K_PUSH = 0, ZC1_K_SORT, ZC1_K_FIELDS, ZC1_NKIND };
ZC_API zc_status zc1_set_profile(zc1_sim *sim, int on);
ZC_API zc_status zc1_get_profile(zc1_sim *sim, double ms[ZC1_NKIND], long long launches[ZC1_NKIND]);
/* field energy per component (emf_get_energy, em1d/emf.c:590-612) and each
 * species' time-centred kinetic energy of its last advance */
ZC_API zc_status zc1_energy(zc1_sim *sim, double emf_energy[6], double *kin_energy);
ZC_API zc_status zc1_species_count(zc1_sim *sim, int species, int *np);
ZC_API zc_status zc1_get_particles(zc1_sim *sim, int species, zc1_part *out, int cap, int *np);
ZC_API zc_status zc1_get_info(zc1_sim *sim, int *iter, int *n_move);
ZC_API zc_status zc_set_current(zc_sim *sim, const float *J_buf);
/* field energy per component (emf_get_energy, em2d/emf.c:729-750) and the
 * time-centred kinetic energy of each species after its last advance
 * (spec->energy, em2d/particles.c:1231); FP64 reductions on the device */
ZC_API zc_status zc_energy(zc_sim *sim, double emf_energy[6], double *kin_energy);
/* zc_energy without the wait: the reductions and the copies into the two
 * host arrays are queued behind the work already queued, and the arrays
 * hold the values once zc_synchronize (or any waiting call) returns.  A run
 * that reports energies every step then never idles the device between
 * steps.  With page-locked arrays the device writes them itself and they
 * must stay allocated until that wait; other host memory is filled before
 * the call returns. */
ZC_API zc_status zc_energy_async(zc_sim *sim, double emf_energy[6], double *kin_energy);
/* charge density of one species on an (nx+1)*(ny+1) grid
 * (spec_deposit_charge, em2d/particles.c:1289-1324) */
ZC_API zc_status zc_species_charge(zc_sim *sim, int species, float *charge);
/* phase-space density of one species added to `buf` (pha_nx[0]*pha_nx[1]
 * floats, host memory): quantities 1 x1, 2 x2, 4 u1, 5 u2, 6 u3 as the
 * reference's rep_type nibbles; pha_range = {x1min, x1max, x2min, x2max}
 * (spec_deposit_pha, em2d/particles.c:1569-1632) */
ZC_API zc_status zc_species_phasespace(zc_sim *sim, int species, int quant1, int quant2, const int pha_nx[2],
                                       const float pha_range[4], float *buf);
ZC_API zc_status zc_get_info(zc_sim *sim, zc_info *info);
ZC_API zc_status zc_grid_view_get(zc_sim *sim, zc_grid_view *view);
ZC_API zc_status zc_synchronize(zc_sim *sim);
/* device time (ms) of the last zc_step / phase call, CUDA events */
ZC_API zc_status zc_last_step_ms(zc_sim *sim, float *ms);

/* --- per-phase device timing ------------------------------------------- */
/* With profiling on (zc_set_profiling 1), every phase of the step is
 * bracketed by CUDA events on the handle's stream; with 2, only the push
 * (ZC_PHASE_PUSH), so that the rest of the step runs as without profiling.
 * zc_get_profile returns, per phase, the summed device milliseconds and the
 * number of kernel launches since the last reset.  The reference's own
 * counters are wall-clock totals of spec_advance and emf_advance
 * (em2d/particles.c:26-59, em2d/emf.c:27-37). */
enum {
    ZC_PHASE_PUSH = 0,      /* fused push + deposit, one CTA per tile */
    ZC_PHASE_SPILL,         /* push of particles outside the tiles */
    ZC_PHASE_MIGRATE,       /* tile migration */
    ZC_PHASE_KIN_ENERGY,    /* kinetic-energy reduction */
    ZC_PHASE_ZERO,          /* current zeroing */
    ZC_PHASE_FOLD,          /* current guard-cell fold */
    ZC_PHASE_SMOOTH,        /* current filter passes */
    ZC_PHASE_YEE,           /* fused Yee advance */
    ZC_PHASE_EMF_GC,        /* field guard cells */
    ZC_PHASE_EXT,           /* external fields */
    ZC_PHASE_WINDOW,        /* moving-window shift and injection */
    ZC_PHASE_SORT,          /* per-tile cell sort */
    ZC_PHASE_HISTORY,       /* per-step energy history */
    ZC_NPHASE
};
ZC_API zc_status zc_set_profiling(zc_sim *sim, int mode);  /* 0 off, 1 every phase, 2 the push only */
ZC_API zc_status zc_get_profile(zc_sim *sim, double ms[ZC_NPHASE], long long launches[ZC_NPHASE]);
ZC_API zc_status zc_reset_profile(zc_sim *sim);
ZC_API const char *zc_phase_name(int phase);

/* --- graph replay ---------------------------------------------------------- */
/* With graphs on, zc_step runs whole blocks of steps (2 x sort_every steps,
 * or 2 with sorting off) as one captured CUDA graph, with eager steps up to
 * the first block boundary and after the last whole block.  Results are
 * those of eager steps.  Not used with a moving window (its injection calls
 * back into the host) or while profiling.  Any change of layout or
 * configuration recaptures the block.  Off by default.  No counterpart in
 * the reference (its step is a host loop, em2d/simulation.c:45-56). */
ZC_API zc_status zc_set_graphs(zc_sim *sim, int enable);

/* --- per-step energy history -------------------------------------------- */
/* Records, after every step, one row of 6 + n_species doubles on the
 * device: the field energy per component (as zc_energy) and the kinetic
 * energy of each species, for up to `max_steps` steps (later steps are not
 * recorded).  The rows the reference's sim_report_energy prints once per
 * call (em2d/simulation.c:183-205) become a device array read once at the
 * end.  Species must be created first.  max_steps = 0 turns it off. */
ZC_API zc_status zc_history_enable(zc_sim *sim, int max_steps);
/* the same rows written by the device straight into the caller's
 * page-locked host memory (`rows`, max_steps * (6 + n_species) doubles,
 * cudaHostAlloc'd): every step's energies reach the host as the step ends,
 * with no copy call, also inside replayed graphs.  The rows hold their values
 * once zc_synchronize (or any waiting call) returns; zc_history_get reads the
 * count.  The rows must stay allocated while the history streams into them.
 * rows = NULL with max_steps = 0 turns it off. */
ZC_API zc_status zc_history_stream(zc_sim *sim, double *rows, int max_steps);
/* copies up to `cap_rows` rows into `out` (row-major); *nrows receives the
 * rows recorded, *ncols the row length.  out == NULL only queries. */
ZC_API zc_status zc_history_get(zc_sim *sim, double *out, int cap_rows, int *nrows, int *ncols);
ZC_API zc_status zc_history_reset(zc_sim *sim);

/* --- batched runs (parameter scans) ---------------------------------------- */
/* A batch advances many independent simulations together: one CUDA graph
 * holds a block of steps of every member of a group as parallel branches,
 * so small grids that cannot fill the GPU alone share it, and one launch per
 * block and group replaces hundreds.  Members keep their own handles (data
 * access, energy, history) and must share the block length (same
 * sort_every) and have no moving window.  Replaces the reference's
 * process-level fan-out of a parameter scan
 * (mods/em1d_param_scan/main.c:112-133); each member gives the results it
 * gives alone. */
typedef struct zc_batch zc_batch;
ZC_API zc_status zc_batch_create(zc_sim *const *sims, int nsims, zc_batch **out);
/* The members are dealt into groups of about equal particle capacity, each
 * with its own stream and graphs: a group's first block starts as soon as
 * its own graph is recorded, and groups do not wait for one another between
 * blocks.  By default one group per 32 members (1 to 8); ngroups <= 0
 * restores that, larger counts are capped at the member count.  Results do
 * not depend on the grouping. */
ZC_API zc_status zc_batch_set_groups(zc_batch *batch, int ngroups);
ZC_API zc_status zc_batch_get_groups(zc_batch *batch, int *ngroups);
/* advances every member by nsteps */
ZC_API zc_status zc_batch_step(zc_batch *batch, int nsteps);
/* device time (ms) of the last zc_batch_step, CUDA events */
ZC_API zc_status zc_batch_last_ms(zc_batch *batch, float *ms);
ZC_API zc_status zc_batch_destroy(zc_batch *batch);

/* --- differentiable step (adjoint) --------------------------------------- */
/* A forward engine of the em2d step with a charge weight per particle, and
 * its hand-written reverse: the gradient of an objective of the fields after
 * the last step with respect to every particle's weight, initial position
 * and momentum, and the initial E and B.  Periodic, or with a moving window
 * (absorbing x edges, x guard cells with the reference's Yee ranges, the
 * window shift, particles entering at their birth step); current filter
 * passes along x.  Objectives: 0 the total field energy (the sum of
 * emf_get_energy's components, em2d/emf.c:729-750); 1 dx sum Ex^2 along one
 * row of cells, over a range of columns (an on-axis wake amplitude).
 * The reverse sweep recomputes the forward run from checkpoints kept every
 * `checkpoint_every` steps.  Float32 (the reference's arithmetic) or float64
 * (for finite-difference checks).  No counterpart in the reference, whose
 * charge is species-wide (em2d/particles.c:557,576). */
typedef struct zc_adj zc_adj;
typedef struct {
    int nx[2];
    double box[2];
    double dt;
    double q;               /* charge of a particle of weight 1 (spec->q) */
    double m_q;
    int np;                 /* particles */
    int checkpoint_every;
    int precision;          /* 0 float32, 1 float64 */
    int device;
    int moving_window;      /* 1: moving window (fields [3][ny][nx+3], cells -1 .. nx+1) */
    int objective;          /* 0 field energy, 1 on-axis Ex (row objective_row) */
    int objective_row;
    int objective_cells[2]; /* cells i0 .. i1-1 of the on-axis objective (i1 <= 0: to nx) */
} zc_adj_desc;
ZC_API zc_status zc_adj_create(const zc_adj_desc *desc, zc_adj **out);
ZC_API zc_status zc_adj_destroy(zc_adj *adj);
/* initial state: particle cells and in-cell positions (as t_part), momenta,
 * weights (np each); E and B as 3 planes [component][iy][column] of
 * nx (periodic) or nx+3 (moving window, cell i at column i+1) columns
 * (NULL: zero) */
ZC_API zc_status zc_adj_set_state(zc_adj *adj, const int *ix, const int *iy, const double *x, const double *y,
                                  const double *ux, const double *uy, const double *uz, const double *w,
                                  const double *E, const double *B);
/* runs nsteps from the current state, keeping checkpoints; returns the
 * objective (field energy after the last step) and the kinetic energy of the
 * last step's particles (NULL to skip either) */
ZC_API zc_status zc_adj_forward(zc_adj *adj, int nsteps, double *objective, double *kinetic);
/* gradient of the objective of the last forward run with respect to the
 * initial state (any pointer may be NULL); the engine's state returns to the
 * start of that run */
ZC_API zc_status zc_adj_backward(zc_adj *adj, double *d_w, double *d_x, double *d_y, double *d_ux, double *d_uy,
                                 double *d_uz, double *d_E, double *d_B);
/* current state (after a forward run: its end); alive = 0 for particles that
 * left through an absorbing x edge */
ZC_API zc_status zc_adj_get_state(zc_adj *adj, int *ix, int *iy, int *alive, double *x, double *y, double *ux,
                                  double *uy, double *uz, double *E, double *B);
/* step at which each particle starts (moving-window injection: the step
 * after the window move that uncovers its column); NULL: all at step 0 */
ZC_API zc_status zc_adj_set_birth(zc_adj *adj, const int *birth);
/* current filter passes along x, each [sa, sb, sa] (kernel_x,
 * em2d/current.c:316-354; binomial sa = 1/4, sb = 1/2) */
ZC_API zc_status zc_adj_set_smooth(zc_adj *adj, int npasses, const double *sa, const double *sb);
/* device time (ms) of the last forward and backward calls, CUDA events */
ZC_API zc_status zc_adj_times(zc_adj *adj, float *forward_ms, float *backward_ms);

/* --- field energy without device allocation ----------------------------- */
/* No counterpart in the reference.  Computes the six field-energy components
 * (the first output of zc_energy) of caller-owned device grids -- E and B
 * each as three SoA planes of `plane` floats, rows of `pitch` floats, cell
 * (i, j) at [(j+1)*pitch + i+1], i.e. the layout of zc_grid_view -- into
 * `energy` (6 doubles of device memory), enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream).  It allocates nothing: for
 * callers whose time loop cannot call cudaMalloc/cudaFree (device memory
 * already owned by another allocator, or no room for the synchronisation
 * those calls bring).  Its scratch is a fixed device array of
 * ZC_STATIC_MAX_ROWS rows; larger grids are rejected with ZC_EINVAL.  The
 * first call on a device looks up that array's address, so make it before
 * any stream capture.  The address is kept per device ordinal for the
 * runtime's primary context: callers on another driver-API context of the
 * device, or after a cudaDeviceReset in the process, are not supported.
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised. */
#define ZC_STATIC_MAX_ROWS 8192
ZC_API zc_status zc_field_energy_static(const float *E, const float *B, size_t plane, int pitch, int nx,
                                        int ny, float dx, float dy, double *energy, void *stream);

/* Test hook, no counterpart in the reference: writes the error word that the
 * kernels set on a failed check (ZC_EPARTICLE_ESCAPE, ZC_ETIMEOUT or
 * ZC_EOVERFLOW), between steps, so that the next zc_step reports it exactly
 * as a failure seen on the device; callers exercise their error paths with
 * it without making a kernel fail.  Other statuses: ZC_EINVAL. */
ZC_API zc_status zc_post_device_error(zc_sim *sim, zc_status which);

/* message of the last failing call on this thread */
ZC_API const char *zc_last_error(void);
ZC_API const char *zc_status_string(zc_status s);

#ifdef __cplusplus
}
#endif
#endif
