/*
 * ref_driver.c -- flat C entry points over the UNMODIFIED reference em2d
 * sources, so the tests can drive the reference exactly like the oracle
 * restatement (same function shapes, prefix zr_ instead of zo_).
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with
 * the reference's own em2d/*.c (minus main.c) into oracle/_ref/.  It
 * includes the reference headers from the reference tree; nothing of the
 * reference is copied into this repository.
 *
 * The reference keeps the random generator, the Box-Muller cache and the
 * timers as process globals, so one process drives one simulation at a time.
 */
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include "simulation.h"
#include "random.h"

typedef struct {
    t_simulation sim;
    t_species *spec;
    int nspec;
    int nx[2];
    float box[2];
    float dt;
    int finalized;
} zr_sim;

typedef struct { int ix, iy; float x, y, ux, uy, uz; } zr_part;
typedef struct { float x, y, z; } zr_f3;
typedef float (*zr_density_fn)(float, void *);
typedef struct {
    float n; int type; float start, end;
    zr_density_fn custom_x; void *custom_data_x;
    zr_density_fn custom_y; void *custom_data_y;
} zr_density;
typedef struct {
    int type; float start, fwhm, rise, flat, fall, a0, omega0, polarization, W0, focus, axis;
} zr_laser;

void zr_set_rand_seed(uint32_t w, uint32_t z) { set_rand_seed(w, z); }
double zr_rand_norm(void) { return rand_norm(); }

zr_sim *zr_sim_new(const int nx[2], const float box[2], float dt)
{
    zr_sim *s = (zr_sim *)calloc(1, sizeof(zr_sim));
    s->nx[0] = nx[0]; s->nx[1] = nx[1];
    s->box[0] = box[0]; s->box[1] = box[1];
    s->dt = dt;
    return s;
}

int zr_sim_add_species(zr_sim *s, const char *name, float m_q, const int ppc[2],
                       const float *ufl, const float *uth, const zr_density *dens)
{
    s->spec = (t_species *)realloc(s->spec, (size_t)(s->nspec + 1) * sizeof(t_species));
    t_species *sp = &s->spec[s->nspec];
    memset(sp, 0, sizeof(*sp));
    t_density d, *dp = NULL;
    if (dens) {
        memset(&d, 0, sizeof(d));
        d.n = dens->n; d.type = (enum density_type)dens->type;
        d.start = dens->start; d.end = dens->end;
        d.custom_x = dens->custom_x; d.custom_data_x = dens->custom_data_x;
        d.custom_y = dens->custom_y; d.custom_data_y = dens->custom_data_y;
        dp = &d;
    }
    int ppc_[2] = {ppc[0], ppc[1]};
    spec_new(sp, (char *)(name ? name : "species"), m_q, ppc_, ufl, uth, s->nx, s->box, s->dt, dp);
    return s->nspec++;
}

/* sim_new must see the final species array */
void zr_sim_finalize(zr_sim *s)
{
    if (s->finalized) return;
    sim_new(&s->sim, s->nx, s->box, s->dt, 0.0f, 0, s->spec, s->nspec);
    s->finalized = 1;
}

void zr_sim_delete(zr_sim *s)
{
    if (!s) return;
    if (s->finalized) sim_delete(&s->sim);   /* frees the species array too */
    else {
        for (int k = 0; k < s->nspec; k++) spec_delete(&s->spec[k]);
        free(s->spec);
    }
    free(s);
}

int zr_sim_set_smooth(zr_sim *s, int xtype, int xlevel, int ytype, int ylevel)
{
    t_smooth sm = {(enum smooth_type)xtype, (enum smooth_type)ytype, xlevel, ylevel};
    sim_set_smooth(&s->sim, &sm);
    return 0;
}

void zr_sim_set_moving_window(zr_sim *s) { sim_set_moving_window(&s->sim); }

int zr_sim_add_laser(zr_sim *s, const zr_laser *L)
{
    t_emf_laser l;
    memset(&l, 0, sizeof(l));
    l.type = (enum emf_laser_type)L->type;
    l.start = L->start; l.fwhm = L->fwhm; l.rise = L->rise; l.flat = L->flat; l.fall = L->fall;
    l.a0 = L->a0; l.omega0 = L->omega0; l.polarization = L->polarization;
    l.W0 = L->W0; l.focus = L->focus; l.axis = L->axis;
    sim_add_laser(&s->sim, &l);
    return 0;
}

/* out-pointer callback as seen from ctypes, wrapped into the reference's
 * by-value float3 callback through a trampoline */
typedef void (*zr_field_fn)(int, float, int, float, void *, float *);
typedef struct { zr_field_fn fn; void *data; } zr_tramp;
static zr_tramp g_tramp[4];   /* ext E, ext B, init E, init B */

static float3 zr_call(int slot, int ix, float dx, int iy, float dy)
{
    float o[3] = {0, 0, 0};
    g_tramp[slot].fn(ix, dx, iy, dy, g_tramp[slot].data, o);
    float3 r = {o[0], o[1], o[2]};
    return r;
}
static float3 tr_ext_E(int ix, float dx, int iy, float dy, void *d) { (void)d; return zr_call(0, ix, dx, iy, dy); }
static float3 tr_ext_B(int ix, float dx, int iy, float dy, void *d) { (void)d; return zr_call(1, ix, dx, iy, dy); }
static float3 tr_init_E(int ix, float dx, int iy, float dy, void *d) { (void)d; return zr_call(2, ix, dx, iy, dy); }
static float3 tr_init_B(int ix, float dx, int iy, float dy, void *d) { (void)d; return zr_call(3, ix, dx, iy, dy); }

int zr_sim_set_ext_fld(zr_sim *s, int E_type, const float E0[3], zr_field_fn E_fn, void *E_data,
                       int B_type, const float B0[3], zr_field_fn B_fn, void *B_data)
{
    t_emf_ext_fld f;
    memset(&f, 0, sizeof(f));
    f.E_type = (enum emf_fld_type)E_type;
    f.B_type = (enum emf_fld_type)B_type;
    if (E0) { f.E_0.x = E0[0]; f.E_0.y = E0[1]; f.E_0.z = E0[2]; }
    if (B0) { f.B_0.x = B0[0]; f.B_0.y = B0[1]; f.B_0.z = B0[2]; }
    g_tramp[0].fn = E_fn; g_tramp[0].data = E_data;
    g_tramp[1].fn = B_fn; g_tramp[1].data = B_data;
    f.E_custom = E_fn ? tr_ext_E : NULL;
    f.B_custom = B_fn ? tr_ext_B : NULL;
    sim_set_ext_fld(&s->sim, &f);
    return 0;
}

int zr_sim_init_fld(zr_sim *s, int E_type, const float E0[3], zr_field_fn E_fn, void *E_data,
                    int B_type, const float B0[3], zr_field_fn B_fn, void *B_data)
{
    t_emf_init_fld f;
    memset(&f, 0, sizeof(f));
    f.E_type = (enum emf_fld_type)E_type;
    f.B_type = (enum emf_fld_type)B_type;
    if (E0) { f.E_0.x = E0[0]; f.E_0.y = E0[1]; f.E_0.z = E0[2]; }
    if (B0) { f.B_0.x = B0[0]; f.B_0.y = B0[1]; f.B_0.z = B0[2]; }
    g_tramp[2].fn = E_fn; g_tramp[2].data = E_data;
    g_tramp[3].fn = B_fn; g_tramp[3].data = B_data;
    f.E_custom = E_fn ? tr_init_E : NULL;
    f.B_custom = B_fn ? tr_init_B : NULL;
    emf_init_fld(&s->sim.emf, &f);
    return 0;
}

void zr_sim_iter(zr_sim *s) { sim_iter(&s->sim); }
void zr_current_zero(zr_sim *s) { current_zero(&s->sim.current); }
void zr_spec_advance(zr_sim *s, int k) { spec_advance(&s->spec[k], &s->sim.emf, &s->sim.current); }
void zr_current_update(zr_sim *s) { current_update(&s->sim.current); }
void zr_emf_advance(zr_sim *s) { emf_advance(&s->sim.emf, &s->sim.current); }

/* disables the periodic sort so buffer order is comparable with the oracle */
void zr_spec_set_n_sort(zr_sim *s, int k, int n) { s->spec[k].n_sort = n; }

int zr_nrow(const zr_sim *s) { return s->sim.emf.nrow; }
int zr_buf_cells(const zr_sim *s) { return (s->nx[0] + 3) * (s->nx[1] + 3); }
int zr_n_species(const zr_sim *s) { return s->nspec; }
int zr_spec_np(const zr_sim *s, int k) { return s->spec[k].np; }
float zr_spec_q(const zr_sim *s, int k) { return s->spec[k].q; }
double zr_spec_energy(const zr_sim *s, int k) { return s->spec[k].energy; }
int zr_spec_n_move(const zr_sim *s, int k) { return s->spec[k].n_move; }
int zr_emf_n_move(const zr_sim *s) { return s->sim.emf.n_move; }
int zr_emf_iter(const zr_sim *s) { return s->sim.emf.iter; }

void zr_get_particles(const zr_sim *s, int k, zr_part *out)
{
    memcpy(out, s->spec[k].part, (size_t)s->spec[k].np * sizeof(t_part));
}

void zr_set_particles(zr_sim *s, int k, const zr_part *in, int np)
{
    spec_grow_buffer(&s->spec[k], np);
    memcpy(s->spec[k].part, in, (size_t)np * sizeof(t_part));
    s->spec[k].np = np;
}

static size_t nbytes(const zr_sim *s) { return (size_t)zr_buf_cells(s) * sizeof(float3); }
void zr_get_E(const zr_sim *s, float *b) { memcpy(b, s->sim.emf.E_buf, nbytes(s)); }
void zr_get_B(const zr_sim *s, float *b) { memcpy(b, s->sim.emf.B_buf, nbytes(s)); }
void zr_get_J(const zr_sim *s, float *b) { memcpy(b, s->sim.current.J_buf, nbytes(s)); }
void zr_get_E_part(const zr_sim *s, float *b)
{
    memcpy(b, s->sim.emf.E_part - 1 - s->sim.emf.nrow, nbytes(s));
}
void zr_get_B_part(const zr_sim *s, float *b)
{
    memcpy(b, s->sim.emf.B_part - 1 - s->sim.emf.nrow, nbytes(s));
}
void zr_set_E(zr_sim *s, const float *b) { memcpy(s->sim.emf.E_buf, b, nbytes(s)); }
void zr_set_B(zr_sim *s, const float *b) { memcpy(s->sim.emf.B_buf, b, nbytes(s)); }
void zr_set_J(zr_sim *s, const float *b) { memcpy(s->sim.current.J_buf, b, nbytes(s)); }
void zr_emf_energy(const zr_sim *s, double en[6]) { emf_get_energy(&s->sim.emf, en); }
void zr_spec_charge(const zr_sim *s, int k, float *rho) { spec_deposit_charge(&s->spec[k], rho); }
void zr_spec_pha(const zr_sim *s, int k, int q1, int q2, const int pha_nx[2], const float range[4], float *buf)
{
    const float r[2][2] = {{range[0], range[1]}, {range[2], range[3]}};
    spec_deposit_pha(&s->spec[k], q1 + 16 * q2, pha_nx, r, buf);
}

/* the reference's own ZDF reports (em2d/emf.c:368, current.c:194,
 * particles.c:1725), written below the current directory */
void zr_report_emf(zr_sim *s, int field, int fc) { emf_report(&s->sim.emf, (char)field, fc); }
void zr_report_current(zr_sim *s, int jc) { current_report(&s->sim.current, jc); }
void zr_report_spec(zr_sim *s, int k, int rep_type, const int pha_nx[2], const float range[4])
{
    const float r[2][2] = {{range[0], range[1]}, {range[2], range[3]}};
    spec_report(&s->spec[k], rep_type, pha_nx, r);
}

/* cumulative particle-advance time and pushes (em2d/particles.c:36-59) */
double zr_spec_time(void) { return spec_time(); }
double zr_spec_npush(void) { return (double)spec_npush(); }
