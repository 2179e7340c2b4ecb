/*
 * ref_driver_em1d.c -- flat C entry points over the UNMODIFIED reference
 * em1d sources (prefix zr1_), for the 1-D step's fixtures and tests.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with the
 * reference's own em1d/*.c (minus main.c) into oracle/_ref/.  It includes the
 * reference headers from the reference tree; nothing of the reference is
 * copied into this repository.  One process drives one simulation at a time
 * (the reference keeps its generator and timers in process globals).
 */
#include <stdlib.h>
#include <string.h>

#include "simulation.h"
#include "random.h"

typedef struct {
    t_simulation sim;
    t_species *spec;
    int nspec;
    int nx;
    float box;
    float dt;
} zr1_sim;

typedef struct { int ix; float x, ux, uy, uz; } zr1_part;

void zr1_set_rand_seed(uint32_t w, uint32_t z) { set_rand_seed(w, z); }

zr1_sim *zr1_sim_new(int nx, float box, float dt)
{
    zr1_sim *s = (zr1_sim *)calloc(1, sizeof(zr1_sim));
    s->nx = nx;
    s->box = box;
    s->dt = dt;
    return s;
}

/* density type: the reference's enum (UNIFORM 0, EMPTY 1, STEP 2, SLAB 3) */
int zr1_add_species(zr1_sim *s, const char *name, float m_q, int ppc, const float ufl[3], const float uth[3],
                    int dtype, float start, float end, float n)
{
    s->spec = (t_species *)realloc(s->spec, (size_t)(s->nspec + 1) * sizeof(t_species));
    t_density d;
    memset(&d, 0, sizeof(d));
    d.n = n;
    d.type = (enum density_type)dtype;
    d.start = start;
    d.end = end;
    char nm[MAX_SPNAME_LEN + 1];
    strncpy(nm, name, MAX_SPNAME_LEN);
    nm[MAX_SPNAME_LEN] = 0;
    spec_new(&s->spec[s->nspec], nm, m_q, ppc, ufl, uth, s->nx, s->box, s->dt, &d);
    return s->nspec++;
}

void zr1_finalize(zr1_sim *s) { sim_new(&s->sim, s->nx, s->box, s->dt, 1e9f, 0, s->spec, s->nspec); }

void zr1_sim_delete(zr1_sim *s)
{
    sim_delete(&s->sim);
    free(s);
}

void zr1_set_smooth(zr1_sim *s, int type, int level)
{
    t_smooth sm = {.xtype = (enum smooth_type)type, .xlevel = level};
    sim_set_smooth(&s->sim, &sm);
}

void zr1_set_moving_window(zr1_sim *s) { sim_set_moving_window(&s->sim); }

/* open boundaries: Mur fields, absorbed particles (the field and particle
 * settings of the reference's input decks, e.g. em1d/input/absorbing.c) */
void zr1_set_open(zr1_sim *s, int fields, int particles)
{
    if (fields) s->sim.emf.bc_type = EMF_BC_OPEN;
    if (particles)
        for (int k = 0; k < s->nspec; k++) s->spec[k].bc_type = PART_BC_OPEN;
}

void zr1_add_laser(zr1_sim *s, float start, float fwhm, float a0, float omega0, float polarization)
{
    t_emf_laser L;
    memset(&L, 0, sizeof(L));
    L.start = start;
    L.fwhm = fwhm;
    L.a0 = a0;
    L.omega0 = omega0;
    L.polarization = polarization;
    sim_add_laser(&s->sim, &L);
}

void zr1_iter(zr1_sim *s) { sim_iter(&s->sim); }
int zr1_spec_np(const zr1_sim *s, int k) { return s->spec[k].np; }
float zr1_spec_q(const zr1_sim *s, int k) { return s->spec[k].q; }
double zr1_spec_energy(const zr1_sim *s, int k) { return s->spec[k].energy; }
int zr1_n_move(const zr1_sim *s) { return s->sim.emf.n_move; }
void zr1_set_n_sort(zr1_sim *s, int k, int n) { s->spec[k].n_sort = n; }

void zr1_get_particles(const zr1_sim *s, int k, zr1_part *out)
{
    memcpy(out, s->spec[k].part, (size_t)s->spec[k].np * sizeof(zr1_part));
}

static size_t nbytes(const zr1_sim *s) { return (size_t)(s->nx + 3) * sizeof(float3); }
void zr1_get_E(const zr1_sim *s, float *b) { memcpy(b, s->sim.emf.E_buf, nbytes(s)); }
void zr1_get_B(const zr1_sim *s, float *b) { memcpy(b, s->sim.emf.B_buf, nbytes(s)); }
void zr1_get_J(const zr1_sim *s, float *b) { memcpy(b, s->sim.current.J_buf, nbytes(s)); }
void zr1_emf_energy(const zr1_sim *s, double en[6]) { emf_get_energy(&s->sim.emf, en); }
