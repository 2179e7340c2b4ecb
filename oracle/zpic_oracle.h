/*
 * zpic_oracle.h -- CPU restatement of the ZPIC em2d electromagnetic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only the test-suite, the smoke check and the CPU-baseline leg of the
 * benchmark may load it.  The product (libzpic_cuda / zpic_gb300) never
 * links or calls it.
 *
 * It restates, in plain C99 with strict IEEE float32 arithmetic (compile with
 * -O2 -fno-fast-math -ffp-contract=off), the reference algorithms of
 *   em2d/random.c      (MWC generator + polar Box-Muller)
 *   em2d/particles.c   (injection, Boris push, zigzag deposit, boundaries,
 *                       moving window)
 *   em2d/current.c     (guard-cell fold, binomial / compensated smoothing)
 *   em2d/emf.c         (Yee solver, guard cells, moving window, laser,
 *                       external fields, field energy)
 *   em2d/simulation.c  (sim_iter ordering, Courant check)
 * Every function cites the reference file:line it follows.  The oracle is
 * pinned bit-for-bit against the reference itself (compiled from its own
 * sources by oracle/build_ref.sh) and against the committed golden vectors in
 * tests/golden/.
 *
 * Grids use the reference layout: float3 interleaved, (nx+3)*(ny+3) cells,
 * guard cells 1 below and 2 above in each direction, row stride nrow = nx+3,
 * cell (0,0) at buffer offset 1 + nrow.
 */
#ifndef ZPIC_ORACLE_H
#define ZPIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Particle record, same 28-byte layout as t_part (em2d/particles.h:29-37). */
typedef struct {
    int ix, iy;
    float x, y;
    float ux, uy, uz;
} zo_part;

typedef struct { float x, y, z; } zo_f3;

/* Density profile kinds, same numbering as enum density_type
 * (em2d/particles.h:43-49). */
enum { ZO_UNIFORM = 0, ZO_EMPTY = 1, ZO_STEP = 2, ZO_SLAB = 3, ZO_CUSTOM = 4 };

/* Smoothing kinds, same numbering as enum smooth_type (em2d/current.h:19-23). */
enum { ZO_SMOOTH_NONE = 0, ZO_SMOOTH_BINOMIAL = 1, ZO_SMOOTH_COMPENSATED = 2 };

/* External / initial field kinds (em2d/emf.h:20-24). */
enum { ZO_FLD_NONE = 0, ZO_FLD_UNIFORM = 1, ZO_FLD_CUSTOM = 2 };

typedef float (*zo_density_fn)(float, void *);
/* custom field callback: (ix, dx, iy, dy, user data, out[3]); the reference's
 * by-value float3 return (em2d/emf.h:40-41) is passed through out[] so that
 * ctypes callbacks can supply it */
typedef void (*zo_field_fn)(int, float, int, float, void *, float *);

typedef struct {
    float n;
    int type;
    float start, end;
    zo_density_fn custom_x;
    void *custom_data_x;
    zo_density_fn custom_y;
    void *custom_data_y;
} zo_density;

typedef struct {
    int type;               /* 0 plane, 1 gaussian (em2d/emf.h enum emf_laser_type) */
    float start, fwhm, rise, flat, fall;
    float a0, omega0, polarization;
    float W0, focus, axis;
} zo_laser;

typedef struct zo_sim zo_sim;

/* ---- random numbers (em2d/random.c) ---- */
void zo_set_rand_seed(uint32_t w, uint32_t z);
uint32_t zo_rand_uint32(void);
double zo_rand_norm(void);
/* drops the cached Box-Muller deviate: the generator state of a fresh process */
void zo_rand_fresh(void);

/* ---- simulation object ---- */
/* Returns NULL and fills err when the Courant condition fails
 * (em2d/simulation.c:105-110). */
zo_sim *zo_sim_new(const int nx[2], const float box[2], float dt, char *err, int errlen);
void zo_sim_delete(zo_sim *s);

/* spec_new (em2d/particles.c:535-612): injects the initial distribution with
 * the process-global generator.  Returns the species index. */
int zo_sim_add_species(zo_sim *s, const char *name, float m_q, const int ppc[2],
                       const float *ufl, const float *uth, const zo_density *dens);

int zo_sim_set_smooth(zo_sim *s, int xtype, int xlevel, int ytype, int ylevel);
void zo_sim_set_moving_window(zo_sim *s);
int zo_sim_add_laser(zo_sim *s, const zo_laser *laser);
int zo_sim_set_ext_fld(zo_sim *s, int E_type, const float E0[3], zo_field_fn E_fn, void *E_data,
                       int B_type, const float B0[3], zo_field_fn B_fn, void *B_data);
int zo_sim_init_fld(zo_sim *s, int E_type, const float E0[3], zo_field_fn E_fn, void *E_data,
                    int B_type, const float B0[3], zo_field_fn B_fn, void *B_data);

/* one full step, sim_iter (em2d/simulation.c:45-56) */
void zo_sim_iter(zo_sim *s);
/* the phases of the step, in sim_iter order */
void zo_current_zero(zo_sim *s);
void zo_spec_advance(zo_sim *s, int species);
void zo_current_update(zo_sim *s);
void zo_emf_advance(zo_sim *s);

/* ---- accessors ---- */
int zo_nrow(const zo_sim *s);
int zo_buf_cells(const zo_sim *s);           /* (nx+3)*(ny+3) */
int zo_n_species(const zo_sim *s);
int zo_spec_np(const zo_sim *s, int sp);
float zo_spec_q(const zo_sim *s, int sp);
double zo_spec_energy(const zo_sim *s, int sp);
int zo_spec_n_move(const zo_sim *s, int sp);
int zo_emf_n_move(const zo_sim *s);
int zo_emf_iter(const zo_sim *s);
void zo_get_particles(const zo_sim *s, int sp, zo_part *out);
/* replaces the particle buffer of a species (used to start the oracle and the
 * GPU path from identical particles) */
void zo_set_particles(zo_sim *s, int sp, const zo_part *in, int np);
void zo_get_E(const zo_sim *s, float *buf);   /* buf: 3*buf_cells floats */
void zo_get_B(const zo_sim *s, float *buf);
void zo_get_J(const zo_sim *s, float *buf);
void zo_get_E_part(const zo_sim *s, float *buf);
void zo_get_B_part(const zo_sim *s, float *buf);
void zo_set_E(zo_sim *s, const float *buf);
void zo_set_B(zo_sim *s, const float *buf);
void zo_set_J(zo_sim *s, const float *buf);
/* emf_get_energy (em2d/emf.c:729-750) */
void zo_emf_energy(const zo_sim *s, double energy[6]);
/* spec_deposit_charge (em2d/particles.c:1289-1324): charge grid (nx+1)*(ny+1) */
void zo_spec_charge(const zo_sim *s, int sp, float *charge);
/* spec_deposit_pha (em2d/particles.c:1569-1632): quantities 1 x1, 2 x2,
 * 4 u1, 5 u2, 6 u3; range {x1min, x1max, x2min, x2max}; adds into buf */
void zo_spec_pha(const zo_sim *s, int sp, int q1, int q2, const int pha_nx[2], const float range[4], float *buf);

#ifdef __cplusplus
}
#endif
#endif
