/*
 * em1d_host.c -- libzpic_em1d: ZPIC's em1d C API (include/em1d/*.h) on top
 * of the 1-D GPU step of libzpic_cuda (zc1_*).
 *
 * What runs here, on the host, in plain C99:
 *   - the multiply-with-carry generator and polar Box-Muller deviates
 *     (em1d/random.c), so that particle loading draws the same numbers in
 *     the same order as the reference;
 *   - particle loading (spec_new and its helpers, em1d/particles.c:72-589)
 *     into the species' host buffer in the reference record layout;
 *   - lasers and initial fields on the host field mirrors (emf_add_laser,
 *     emf_init_fld, em1d/emf.c:157-260, 626-680), the parameter checks and
 *     exit(-1) behaviour of the reference;
 *   - the reports (ZDF files through zdf_io.c) from the host mirrors, which
 *     are refreshed from the GPU first.
 * The steps (push, deposit, boundaries, window, current update, field
 * advance) run on the GPU: the first step creates a zc1 simulation from the
 * mirrors, and every step after it is one zc1_step_async.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include "../../../include/em1d/simulation.h"
#include "../../../include/em1d/zdf.h"
#include "../../../include/em1d/random.h"
#include "../../../include/em1d/timer.h"
#include "../../../include/zpic_cuda.h"

#define EXPORT __attribute__((visibility("default")))

static void die(const char *what)
{
    fprintf(stderr, "%s\n", what);
    exit(-1);
}

static void zc_check(zc_status st, const char *where)
{
    if (st != ZC_OK) {
        fprintf(stderr, "(*error*) %s: %s (%s)\n", where, zc_status_string(st), zc_last_error());
        exit(-1);
    }
}

/* ------------------------------------------------------------------------- */
/* timers (em1d/timer.c)                                                     */
/* ------------------------------------------------------------------------- */
EXPORT uint64_t timer_ticks(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return ((uint64_t)tv.tv_sec) * 1000000 + (uint64_t)tv.tv_usec;
}
EXPORT double timer_interval_seconds(uint64_t start, uint64_t end) { return (end - start) * 1.0e-6; }
EXPORT double timer_cpu_seconds(void) { return (double)clock() / CLOCKS_PER_SEC; }
EXPORT double timer_resolution(void) { return 1.0e-6; }

/* ------------------------------------------------------------------------- */
/* random numbers: multiply-with-carry pair and polar Box-Muller (random.c)  */
/* ------------------------------------------------------------------------- */
static uint32_t g_w = 12345, g_z = 67890;  /* the reference's default seeds */
static int g_spare_ok = 0;
static double g_spare = 0.0;

EXPORT void set_rand_seed(uint32_t w, uint32_t z)
{
    /* the cached deviate is kept, as in the reference */
    g_w = w;
    g_z = z;
}

EXPORT void rand_seed_fresh(uint32_t w, uint32_t z)
{
    g_w = w;
    g_z = z;
    g_spare_ok = 0;
    g_spare = 0.0;
}

EXPORT uint32_t rand_uint32(void)
{
    g_z = 36969u * (g_z & 65535u) + (g_z >> 16);
    g_w = 18000u * (g_w & 65535u) + (g_w >> 16);
    return (g_z << 16) + g_w;
}

EXPORT double rand_norm(void)
{
    if (g_spare_ok) {
        g_spare_ok = 0;
        return g_spare;
    }
    double a, b, r2;
    do {
        a = (rand_uint32() + 0.5) / 2147483649.0 - 1.0;
        b = (rand_uint32() + 0.5) / 2147483649.0 - 1.0;
        r2 = a * a + b * b;
    } while (r2 == 0.0 || r2 >= 1.0);
    const double f = sqrt(-2.0 * log(r2) / r2);
    g_spare = a * f;
    g_spare_ok = 1;
    return b * f;
}

/* ------------------------------------------------------------------------- */
/* registry: the GPU simulation behind each t_simulation                     */
/* ------------------------------------------------------------------------- */
typedef struct {
    t_simulation *sim;
    zc1_sim *gpu;
    int pending;     /* steps enqueued since the last wait */
    double step_s;   /* wall time spent in steps and waits */
} entry_t;

#define MAX_SIMS 256
static entry_t *g_reg[MAX_SIMS];

static entry_t *reg_add(t_simulation *sim)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (!g_reg[k]) {
            entry_t *e = (entry_t *)calloc(1, sizeof(entry_t));
            if (!e) die("(*error*) out of memory");
            e->sim = sim;
            g_reg[k] = e;
            return e;
        }
    die("(*error*) too many simulations at once");
    return NULL;
}

static void reg_remove(entry_t *e)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k] == e) g_reg[k] = NULL;
    free(e);
}

static entry_t *reg_by_sim(const t_simulation *sim)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k] && g_reg[k]->sim == sim) return g_reg[k];
    return NULL;
}

static entry_t *reg_by_emf(const t_emf *emf)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k] && &g_reg[k]->sim->emf == emf) return g_reg[k];
    return NULL;
}

static entry_t *reg_by_current(const t_current *current)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k] && &g_reg[k]->sim->current == current) return g_reg[k];
    return NULL;
}

/* the simulation owning species `spec`, and its index there */
static entry_t *reg_by_species(const t_species *spec, int *idx)
{
    for (int k = 0; k < MAX_SIMS; k++) {
        entry_t *e = g_reg[k];
        if (!e || !e->sim->species) continue;
        /* an address range test (subtracting pointers into different
         * arrays is not defined in C) */
        const uintptr_t a = (uintptr_t)spec, lo = (uintptr_t)e->sim->species;
        const uintptr_t hi = lo + (uintptr_t)e->sim->n_species * sizeof(t_species);
        if (a >= lo && a < hi && (a - lo) % sizeof(t_species) == 0) {
            if (idx) *idx = (int)((a - lo) / sizeof(t_species));
            return e;
        }
    }
    return NULL;
}

/* ------------------------------------------------------------------------- */
/* particle loading (em1d/particles.c:72-589)                                */
/* ------------------------------------------------------------------------- */
EXPORT void spec_grow_buffer(t_species *spec, const int size)
{
    if (size > spec->np_max) {
        spec->np_max = (size / 1024 + 1) * 1024;
        spec->part = (t_part *)realloc(spec->part, (size_t)spec->np_max * sizeof(t_part));
        if (!spec->part) die("(*error*) out of memory");
    }
}

/* appends a particle at cell ix, offset x (momenta set by set_u) */
static void put(t_species *spec, int *ip, int ix, float x)
{
    if (*ip >= spec->np_max) spec_grow_buffer(spec, *ip + 1);
    spec->part[*ip].ix = ix;
    spec->part[*ip].x = x;
    *ip += 1;
}

/* thermal momenta with the mean of every cell removed, plus the fluid
 * momentum, for particles start..end (spec_set_u, particles.c:72-135) */
static void set_u(t_species *spec, int start, int end)
{
    for (int i = start; i <= end; i++) {
        spec->part[i].ux = spec->uth[0] * rand_norm();
        spec->part[i].uy = spec->uth[1] * rand_norm();
        spec->part[i].uz = spec->uth[2] * rand_norm();
    }
    float3 *net = (float3 *)calloc((size_t)spec->nx, sizeof(float3));
    int *cnt = (int *)calloc((size_t)spec->nx, sizeof(int));
    if (!net || !cnt) die("(*error*) out of memory");
    for (int i = start; i <= end; i++) {
        const int c = spec->part[i].ix;
        net[c].x += spec->part[i].ux;
        net[c].y += spec->part[i].uy;
        net[c].z += spec->part[i].uz;
        cnt[c] += 1;
    }
    for (int c = 0; c < spec->nx; c++) {
        const float norm = (cnt[c] > 0) ? 1.0f / cnt[c] : 0;
        net[c].x *= norm;
        net[c].y *= norm;
        net[c].z *= norm;
    }
    for (int i = start; i <= end; i++) {
        const int c = spec->part[i].ix;
        spec->part[i].ux += spec->ufl[0] - net[c].x;
        spec->part[i].uy += spec->ufl[1] - net[c].y;
        spec->part[i].uz += spec->ufl[2] - net[c].z;
    }
    free(cnt);
    free(net);
}

/* particle positions in cells range[0]..range[1] by the density profile
 * (spec_set_x, particles.c:250-447) */
static void set_x(t_species *spec, const int range[2])
{
    const int npc = spec->ppc;
    float *poscell = (float *)malloc(sizeof(float) * (size_t)npc);
    if (!poscell) die("(*error*) out of memory");
    for (int k = 0; k < npc; k++) poscell[k] = (k + 0.5) / npc;
    int ip = spec->np;
    const t_density *D = &spec->density;
    switch (D->type) {
    case STEP: {
        const float start = D->start / spec->dx - spec->n_move;
        for (int i = range[0]; i <= range[1]; i++)
            for (int k = 0; k < npc; k++)
                if (i + poscell[k] > start) put(spec, &ip, i, poscell[k]);
        break;
    }
    case SLAB: {
        const float start = D->start / spec->dx - spec->n_move;
        const float end = D->end / spec->dx - spec->n_move;
        for (int i = range[0]; i <= range[1]; i++)
            for (int k = 0; k < npc; k++)
                if (i + poscell[k] > start && i + poscell[k] < end) put(spec, &ip, i, poscell[k]);
        break;
    }
    case RAMP: {
        /* particles spaced so that each carries 1/ppc of the ramp's charge,
         * positions by inverting the linear cumulative density */
        double r0 = D->start / spec->dx;
        const double r1 = D->end / spec->dx;
        if ((range[0] + spec->n_move) > r1 || (range[1] + spec->n_move) < r0) break;
        double n0 = D->ramp[0];
        const double n1 = D->ramp[1];
        if (r0 < 0) {
            n0 += -r0 * (n1 - n0) / (r1 - r0);
            r0 = 0;
        }
        const double cpp = 1.0 / spec->ppc;
        for (unsigned long k = D->total_np_inj;; k++) {
            const double Rs = (k + 0.5) * cpp / (r1 - r0);
            double pos = 2 * Rs / (sqrt(n0 * n0 + 2 * (n1 - n0) * Rs) + n0);
            if (pos > 1) break;
            pos = r0 + (r1 - r0) * pos;
            const int ix = pos;
            if (ix - spec->n_move < range[0]) {
                fprintf(stderr, "(*error*) attempting to inject outside of valid range.\n");
                break;
            }
            if (ix - spec->n_move > range[1]) break;
            put(spec, &ip, ix - spec->n_move, pos - ix);
        }
        break;
    }
    case CUSTOM: {
        /* cumulative density integrated with the trapezoidal rule on the
         * cell edges, particles where it crosses (k + 1/2)/ppc */
        const double dx = spec->dx;
        const double cpp = 1.0 / spec->ppc;
        unsigned long k = D->total_np_inj;
        int ix = range[0];
        double n0;
        double n1 = (*D->custom)((ix + spec->n_move) * dx, D->custom_data);
        double d0;
        double d1 = D->custom_q_inj;
        double Rs;
        while (ix <= range[1]) {
            n0 = n1;
            n1 = (*D->custom)((ix + 1 + spec->n_move) * dx, D->custom_data);
            d0 = d1;
            d1 += 0.5 * (n0 + n1);
            while ((Rs = (k + 0.5) * cpp) < d1) {
                const double pos = 2 * (Rs - d0) / (sqrt(n0 * n0 + 2 * (n1 - n0) * (Rs - d0)) + n0);
                put(spec, &ip, ix, pos);
                k++;
            }
            ix++;
        }
        spec->density.custom_q_inj = d1;
        break;
    }
    case EMPTY:
        break;
    default:
        for (int i = range[0]; i <= range[1]; i++)
            for (int k = 0; k < npc; k++) put(spec, &ip, i, poscell[k]);
    }
    free(poscell);
    spec->density.total_np_inj += ip - spec->np;
    spec->np = ip;
}

static void inject(t_species *spec, const int range[2])
{
    const int start = spec->np;
    set_x(spec, range);
    set_u(spec, start, spec->np - 1);
}

EXPORT void spec_new(t_species *spec, char name[], const float m_q, const int ppc, const float ufl[],
                     const float uth[], const int nx, float box, const float dt, t_density *density)
{
    memset(spec, 0, sizeof(*spec));
    strncpy(spec->name, name, MAX_SPNAME_LEN);
    spec->nx = nx;
    spec->ppc = ppc;
    spec->box = box;
    spec->dx = box / nx;
    spec->m_q = m_q;
    spec->q = copysign(1.0f, m_q) / ppc;  /* in double, then rounded (particles.c:529) */
    spec->dt = dt;
    spec->np_max = 0;
    spec->part = NULL;
    if (density) {
        spec->density = *density;
        if (spec->density.n == 0.) spec->density.n = 1.0;
    } else {
        memset(&spec->density, 0, sizeof(spec->density));
        spec->density.type = UNIFORM;
        spec->density.n = 1.0;
    }
    spec->density.total_np_inj = 0;
    spec->density.custom_q_inj = 0.;
    spec->q *= fabsf(spec->density.n);
    for (int i = 0; i < 3; i++) {
        spec->ufl[i] = ufl ? ufl[i] : 0;
        spec->uth[i] = uth ? uth[i] : 0;
    }
    spec->iter = 0;
    spec->moving_window = 0;
    spec->n_move = 0;
    spec->np = 0;
    const int range[2] = {0, nx - 1};
    inject(spec, range);
    spec->n_sort = 16;
    spec->bc_type = PART_BC_PERIODIC;
}

EXPORT void spec_delete(t_species *spec)
{
    free(spec->part);
    spec->part = NULL;
    spec->np = -1;
}

/* ------------------------------------------------------------------------- */
/* fields and current: host mirrors (em1d/emf.c:49-105, current.c:31-90)     */
/* ------------------------------------------------------------------------- */
EXPORT void emf_new(t_emf *emf, int nx, float box, const float dt)
{
    memset(emf, 0, sizeof(*emf));
    emf->gc[0] = 1;
    emf->gc[1] = 2;
    const size_t n = (size_t)(emf->gc[0] + nx + emf->gc[1]);
    emf->E_buf = (float3 *)calloc(n, sizeof(float3));
    emf->B_buf = (float3 *)calloc(n, sizeof(float3));
    if (!emf->E_buf || !emf->B_buf) die("(*error*) out of memory");
    emf->E = emf->E_buf + emf->gc[0];
    emf->B = emf->B_buf + emf->gc[0];
    emf->nx = nx;
    emf->box = box;
    emf->dx = box / nx;
    emf->dt = dt;
    emf->iter = 0;
    emf->moving_window = 0;
    emf->n_move = 0;
    emf->bc_type = EMF_BC_PERIODIC;
    emf->ext_fld.E_type = EMF_FLD_TYPE_NONE;
    emf->ext_fld.B_type = EMF_FLD_TYPE_NONE;
    emf->E_part = emf->E;
    emf->B_part = emf->B;
}

EXPORT void emf_delete(t_emf *emf)
{
    free(emf->E_buf);
    free(emf->B_buf);
    emf->E_buf = emf->B_buf = NULL;
    emf->E_part = emf->B_part = NULL;
}

EXPORT void current_new(t_current *current, int nx, float box, float dt)
{
    memset(current, 0, sizeof(*current));
    current->gc[0] = 1;
    current->gc[1] = 2;
    current->J_buf = (float3 *)calloc((size_t)(current->gc[0] + nx + current->gc[1]), sizeof(float3));
    if (!current->J_buf) die("(*error*) out of memory");
    current->nx = nx;
    current->J = current->J_buf + current->gc[0];
    current->box = box;
    current->dx = box / nx;
    current->smooth.xtype = NONE;
    current->smooth.xlevel = 0;
    current->iter = 0;
    current->dt = dt;
    current->bc_type = CURRENT_BC_PERIODIC;
}

EXPORT void current_delete(t_current *current)
{
    free(current->J_buf);
    current->J_buf = current->J = NULL;
}

/* periodic guard cells of the field mirrors (emf_update_gc, emf.c:470-500):
 * -1 <- nx-1 and nx <- 0 */
static void mirror_gc(t_emf *emf)
{
    if (emf->bc_type != EMF_BC_PERIODIC) return;
    const int nx = emf->nx;
    emf->E[-1] = emf->E[nx - 1];
    emf->B[-1] = emf->B[nx - 1];
    emf->E[nx] = emf->E[0];
    emf->B[nx] = emf->B[0];
}

/* sin^2 rise and fall around a flat top (lon_env, emf.c:157-180) */
static float lon_env(const t_emf_laser *laser, const float z)
{
    if (z > laser->start) return 0.0;
    if (z > laser->start - laser->rise) {
        const float csi = z - laser->start;
        const float e = sin(M_PI_2 * csi / laser->rise);
        return e * e;
    }
    if (z > laser->start - (laser->rise + laser->flat)) return 1.0;
    if (z > laser->start - (laser->rise + laser->flat + laser->fall)) {
        const float csi = z - (laser->start - laser->rise - laser->flat - laser->fall);
        const float e = sin(M_PI_2 * csi / laser->fall);
        return e * e;
    }
    return 0.0;
}

static void gpu_fields_to_mirror(entry_t *e);
static void mirror_fields_to_gpu(entry_t *e);

EXPORT void emf_add_laser(t_emf *const emf, t_emf_laser *laser)
{
    if (laser->fwhm != 0) {
        if (laser->fwhm <= 0) die("Invalid laser FWHM, must be > 0, aborting.");
        laser->rise = laser->fwhm;
        laser->fall = laser->fwhm;
        laser->flat = 0.;
    }
    if (laser->rise <= 0) die("Invalid laser RISE, must be > 0, aborting.");
    if (laser->flat < 0) die("Invalid laser FLAT, must be >= 0, aborting.");
    if (laser->fall <= 0) die("Invalid laser FALL, must be > 0, aborting.");
    entry_t *e = reg_by_emf(emf);
    if (e && e->gpu) gpu_fields_to_mirror(e);
    float3 *E = emf->E, *B = emf->B;
    const float dx = emf->dx;
    const float amp = laser->omega0 * laser->a0;
    const float cos_pol = cos(laser->polarization);
    const float sin_pol = sin(laser->polarization);
    const float k = laser->omega0;
    for (int i = 0; i < emf->nx; i++) {
        const float z = i * dx;
        const float z_2 = z + dx / 2;
        const float lenv = amp * lon_env(laser, z);
        const float lenv_2 = amp * lon_env(laser, z_2);
        E[i].y += +lenv * cos(k * z) * cos_pol;
        E[i].z += +lenv * cos(k * z) * sin_pol;
        B[i].y += -lenv_2 * cos(k * z_2) * sin_pol;
        B[i].z += +lenv_2 * cos(k * z_2) * cos_pol;
    }
    mirror_gc(emf);
    if (e && e->gpu) mirror_fields_to_gpu(e);
}

EXPORT void emf_init_fld(t_emf *const emf, t_emf_init_fld *init_fld)
{
    if (emf->iter != 0) die("emf_inifloat should only be called at initialization, aborting...");
    const int i0 = -emf->gc[0], i1 = emf->nx + emf->gc[1];
    switch (init_fld->E_type) {
    case EMF_FLD_TYPE_UNIFORM:
        for (int i = i0; i < i1; i++) emf->E[i] = init_fld->E_0;
        break;
    case EMF_FLD_TYPE_CUSTOM:
        for (int i = i0; i < i1; i++) emf->E[i] = (init_fld->E_custom)(i, emf->dx, init_fld->E_custom_data);
        break;
    default:
        break;
    }
    switch (init_fld->B_type) {
    case EMF_FLD_TYPE_UNIFORM:
        for (int i = i0; i < i1; i++) emf->B[i] = init_fld->B_0;
        break;
    case EMF_FLD_TYPE_CUSTOM:
        for (int i = i0; i < i1; i++) emf->B[i] = (init_fld->B_custom)(i, emf->dx, init_fld->B_custom_data);
        break;
    default:
        break;
    }
}

EXPORT void emf_set_ext_fld(t_emf *const emf, t_emf_ext_fld *ext_fld)
{
    (void)emf;
    if (ext_fld->E_type == EMF_FLD_TYPE_NONE && ext_fld->B_type == EMF_FLD_TYPE_NONE) return;
    die("(*error*) external fields are not supported by the 1-D GPU step, aborting.");
}

/* ------------------------------------------------------------------------- */
/* the GPU simulation                                                        */
/* ------------------------------------------------------------------------- */
/* the host record and the C-ABI record are the same 20 bytes */
typedef char part_layout_check[(sizeof(t_part) == sizeof(zc1_part)) ? 1 : -1];

static double g_step_s = 0.0;     /* wall time of the GPU steps, all simulations */
static uint64_t g_npush = 0;      /* particles pushed by finished simulations */

/* counters of the step mirrored into the structs (the GPU keeps every
 * species' counters equal to the field's) */
static void counters_from_gpu(entry_t *e)
{
    int iter = 0, n_move = 0;
    zc_check(zc1_get_info(e->gpu, &iter, &n_move), "sim_iter");
    t_simulation *sim = e->sim;
    sim->emf.iter = iter;
    sim->emf.n_move = n_move;
    sim->current.iter = iter;
    for (int k = 0; k < sim->n_species; k++) {
        sim->species[k].iter = iter;
        sim->species[k].n_move = n_move;
    }
}

/* creates the GPU simulation from what the deck has set up */
static void gpu_create(entry_t *e)
{
    t_simulation *sim = e->sim;
    int n_open = 0;
    for (int k = 0; k < sim->n_species; k++) n_open += sim->species[k].bc_type == PART_BC_OPEN;
    if (n_open && n_open != sim->n_species)
        die("(*error*) the 1-D GPU step takes open boundaries for every species or for none, aborting.");
    zc1_desc d;
    memset(&d, 0, sizeof(d));
    d.nx = sim->emf.nx;
    d.box = sim->emf.box;
    d.dt = sim->emf.dt;
    d.device = 0;
    d.open_fields = sim->emf.bc_type == EMF_BC_OPEN;
    d.open_particles = n_open > 0;
    d.moving_window = sim->emf.moving_window;
    d.sort_every = (sim->n_species > 0 && sim->species[0].n_sort > 0) ? sim->species[0].n_sort : 16;
    zc_check(zc1_create(&d, &e->gpu), "sim_iter");
    for (int k = 0; k < sim->n_species; k++) {
        const t_species *p = &sim->species[k];
        zc1_species_desc sd;
        memset(&sd, 0, sizeof(sd));
        sd.m_q = p->m_q;
        sd.q = p->q;
        sd.ppc = p->ppc;
        for (int c = 0; c < 3; c++) {
            sd.ufl[c] = p->ufl[c];
            sd.uth[c] = p->uth[c];
        }
        switch (p->density.type) {
        case UNIFORM: sd.density = 0; break;
        case STEP: sd.density = 2; break;
        case SLAB: sd.density = 3; break;
        case EMPTY: sd.density = 1; break;
        default:
            if (d.moving_window)
                die("(*error*) moving-window injection on the 1-D GPU step takes uniform, step or slab profiles, "
                    "aborting.");
            sd.density = 1;  /* loaded on the host; nothing is injected without a window */
        }
        sd.start = p->density.start;
        sd.end = p->density.end;
        int id = 0;
        zc_check(zc1_add_species(e->gpu, &sd, (const zc1_part *)p->part, p->np, &id), "sim_iter");
    }
    zc_check(zc1_set_fields(e->gpu, (const float *)sim->emf.E_buf, (const float *)sim->emf.B_buf), "sim_iter");
    if (sim->current.smooth.xtype != NONE)
        zc_check(zc1_set_smooth(e->gpu, (int)sim->current.smooth.xtype, sim->current.smooth.xlevel), "sim_iter");
}

/* waits for the enqueued steps */
static void gpu_wait(entry_t *e)
{
    if (!e->gpu || !e->pending) return;
    const uint64_t t0 = timer_ticks();
    zc_check(zc1_synchronize(e->gpu), "sim_iter");
    e->pending = 0;
    e->step_s += timer_interval_seconds(t0, timer_ticks());
}

static void gpu_fields_to_mirror(entry_t *e)
{
    gpu_wait(e);
    zc_check(zc1_get_fields(e->gpu, (float *)e->sim->emf.E_buf, (float *)e->sim->emf.B_buf), "emf");
}

static void mirror_fields_to_gpu(entry_t *e)
{
    zc_check(zc1_set_fields(e->gpu, (const float *)e->sim->emf.E_buf, (const float *)e->sim->emf.B_buf), "emf");
}

/* one time step of the whole simulation (sim_iter, em1d/simulation.c:45-56) */
static void step(entry_t *e)
{
    if (!e) die("(*error*) unknown simulation (sim_new not called), aborting.");
    const uint64_t t0 = timer_ticks();
    if (!e->gpu) gpu_create(e);
    zc_check(zc1_step_async(e->gpu, 1), "sim_iter");
    e->pending += 1;
    counters_from_gpu(e);
    e->step_s += timer_interval_seconds(t0, timer_ticks());
}

EXPORT void spec_sync_host(t_species *spec)
{
    int k = 0;
    entry_t *e = reg_by_species(spec, &k);
    if (!e || !e->gpu) return;
    gpu_wait(e);
    int n = 0;
    zc_check(zc1_species_count(e->gpu, k, &n), "spec_report");
    spec_grow_buffer(spec, n);
    zc_check(zc1_get_particles(e->gpu, k, (zc1_part *)spec->part, spec->np_max, &n), "spec_report");
    spec->np = n;
    double *kin = (double *)calloc((size_t)e->sim->n_species, sizeof(double));
    if (!kin) die("(*error*) out of memory");
    zc_check(zc1_energy(e->gpu, NULL, kin), "spec_report");
    spec->energy = kin[k];
    free(kin);
}

/* ------------------------------------------------------------------------- */
/* simulation (em1d/simulation.c)                                            */
/* ------------------------------------------------------------------------- */
EXPORT void sim_new(t_simulation *sim, int nx, float box, float dt, float tmax, int ndump, t_species *species,
                    int n_species)
{
    sim->dt = dt;
    sim->tmax = tmax;
    sim->ndump = ndump;
    emf_new(&sim->emf, nx, box, dt);
    current_new(&sim->current, nx, box, dt);
    sim->n_species = n_species;
    sim->species = species;
    const float cour = sim->emf.dx;
    if (dt >= cour) {
        fprintf(stderr, "Invalid timestep, courant condition violation, dtmax = %f \n", cour);
        exit(-1);
    }
    entry_t *old = reg_by_sim(sim);
    if (old) reg_remove(old);
    reg_add(sim);
}

EXPORT void sim_iter(t_simulation *sim) { step(reg_by_sim(sim)); }

EXPORT void sim_add_laser(t_simulation *sim, t_emf_laser *laser) { emf_add_laser(&sim->emf, laser); }

EXPORT void sim_set_moving_window(t_simulation *sim)
{
    entry_t *e = reg_by_sim(sim);
    if (e && e->gpu) die("(*error*) the moving window is set before the first step, aborting.");
    sim->emf.moving_window = 1;
    sim->emf.bc_type = EMF_BC_NONE;
    sim->current.bc_type = CURRENT_BC_NONE;
    for (int i = 0; i < sim->n_species; i++) sim->species[i].moving_window = 1;
}

EXPORT void sim_set_smooth(t_simulation *sim, t_smooth *smooth)
{
    if ((smooth->xtype != NONE) && (smooth->xlevel <= 0)) {
        printf("Invalid smooth level along x direction\n");
        exit(-1);
    }
    sim->current.smooth = *smooth;
    entry_t *e = reg_by_sim(sim);
    if (e && e->gpu) {
        gpu_wait(e);
        zc_check(zc1_set_smooth(e->gpu, (int)smooth->xtype, smooth->xlevel), "sim_set_smooth");
    }
}

EXPORT void sim_set_ext_fld(t_simulation *sim, t_emf_ext_fld *ext_fld) { emf_set_ext_fld(&sim->emf, ext_fld); }

EXPORT int report(int n, int ndump)
{
    if (ndump > 0) return !(n % ndump);
    return 0;
}

/* the phase calls: the GPU step runs all phases at once, in emf_advance */
EXPORT void current_zero(t_current *current) { (void)current; }
EXPORT void current_update(t_current *current) { (void)current; }
EXPORT void spec_advance(t_species *spec, t_emf *emf, t_current *current)
{
    (void)spec;
    (void)emf;
    (void)current;
}
EXPORT void emf_advance(t_emf *emf, const t_current *current)
{
    (void)current;
    step(reg_by_emf(emf));
}

/* ------------------------------------------------------------------------- */
/* energies (emf.c:590-612, simulation.c sim_report_energy)                  */
/* ------------------------------------------------------------------------- */
EXPORT void emf_get_energy(const t_emf *emf, double energy[])
{
    entry_t *e = reg_by_emf(emf);
    if (e && e->gpu) {
        gpu_wait(e);
        zc_check(zc1_energy(e->gpu, energy, NULL), "emf_get_energy");
        return;
    }
    for (int i = 0; i < 6; i++) energy[i] = 0;
    for (int i = 0; i < emf->nx; i++) {
        energy[0] += emf->E[i].x * emf->E[i].x;
        energy[1] += emf->E[i].y * emf->E[i].y;
        energy[2] += emf->E[i].z * emf->E[i].z;
        energy[3] += emf->B[i].x * emf->B[i].x;
        energy[4] += emf->B[i].y * emf->B[i].y;
        energy[5] += emf->B[i].z * emf->B[i].z;
    }
    for (int i = 0; i < 6; i++) energy[i] *= 0.5 * emf->dx;
}

EXPORT void sim_report_energy(t_simulation *sim)
{
    double emf_energy[6];
    emf_get_energy(&sim->emf, emf_energy);
    /* the reference starts the field total from E_x and then adds all six
     * components (simulation.c:155-181); kept as it is */
    double tot_emf = emf_energy[0];
    for (int i = 0; i < 6; i++) tot_emf += emf_energy[i];
    entry_t *e = reg_by_sim(sim);
    if (e && e->gpu && sim->n_species > 0) {
        double *kin = (double *)calloc((size_t)sim->n_species, sizeof(double));
        if (!kin) die("(*error*) out of memory");
        zc_check(zc1_energy(e->gpu, NULL, kin), "sim_report_energy");
        for (int i = 0; i < sim->n_species; i++) sim->species[i].energy = kin[i];
        free(kin);
    }
    double tot_part = 0;
    for (int i = 0; i < sim->n_species; i++) tot_part += sim->species[i].energy;
    printf("Energy (fields | particles | total) = %e %e %e\n", tot_emf, tot_part, tot_emf + tot_part);
}

/* ------------------------------------------------------------------------- */
/* reports (emf.c:268-345, current.c:167-230, particles.c:1093-1490)         */
/* ------------------------------------------------------------------------- */
EXPORT void emf_report(const t_emf *emf, const char field, const int fc)
{
    char vfname[16];
    char vflabel[16];
    const char comp[] = {'x', 'y', 'z'};
    if (fc < 0 || fc > 2) {
        fprintf(stderr, "(*error*) Invalid field component (fc) selected, returning\n");
        return;
    }
    entry_t *e = reg_by_emf(emf);
    if (e && e->gpu) gpu_fields_to_mirror(e);
    const float3 *f;
    switch (field) {
    case EFLD:
        f = emf->E;
        snprintf(vfname, 16, "E%1d", fc);
        snprintf(vflabel, 16, "E_%c", comp[fc]);
        break;
    case BFLD:
        f = emf->B;
        snprintf(vfname, 16, "B%1d", fc);
        snprintf(vflabel, 16, "B_%c", comp[fc]);
        break;
    case EPART:
        f = emf->E_part;
        snprintf(vfname, 16, "E%1d-part", fc);
        snprintf(vflabel, 16, "E_{%cp}", comp[fc]);
        break;
    case BPART:
        f = emf->B_part;
        snprintf(vfname, 16, "B%1d-part", fc);
        snprintf(vflabel, 16, "B_{%cp}", comp[fc]);
        break;
    default:
        fprintf(stderr, "Invalid field type selected, returning\n");
        return;
    }
    float *buf = (float *)malloc(sizeof(float) * (size_t)emf->nx);
    if (!buf) die("(*error*) out of memory");
    for (int i = 0; i < emf->nx; i++) buf[i] = (fc == 0) ? f[i].x : (fc == 1) ? f[i].y : f[i].z;
    t_zdf_grid_axis axis[1];
    memset(axis, 0, sizeof(axis));
    axis[0].min = 0.0 + emf->n_move * emf->dx;
    axis[0].max = emf->box + emf->n_move * emf->dx;
    axis[0].name = "x";
    axis[0].label = "x";
    axis[0].units = "c/\\omega_p";
    t_zdf_grid_info info;
    memset(&info, 0, sizeof(info));
    info.ndims = 1;
    info.name = vfname;
    info.label = vflabel;
    info.units = "m_e c \\omega_p e^{-1}";
    info.axis = axis;
    info.count[0] = emf->nx;
    t_zdf_iteration iter = {.name = "ITERATION", .n = emf->iter, .t = emf->iter * emf->dt,
                            .time_units = "1/\\omega_p"};
    zdf_save_grid(buf, zdf_float32, &info, &iter, "EMF");
    free(buf);
}

EXPORT void current_report(const t_current *current, const int jc)
{
    if (jc < 0 || jc > 2) {
        fprintf(stderr, "(*error*) Invalid current component (jc) selected, returning\n");
        return;
    }
    entry_t *e = reg_by_current(current);
    if (e && e->gpu) {
        gpu_wait(e);
        zc_check(zc1_get_current(e->gpu, (float *)current->J_buf), "current_report");
    }
    float *buf = (float *)malloc(sizeof(float) * (size_t)current->nx);
    if (!buf) die("(*error*) out of memory");
    const float3 *f = current->J;
    for (int i = 0; i < current->nx; i++) buf[i] = (jc == 0) ? f[i].x : (jc == 1) ? f[i].y : f[i].z;
    char vfname[16];
    char vflabel[16];
    snprintf(vfname, 3, "J%1u", (unsigned)jc);
    const char comp[] = {'x', 'y', 'z'};
    snprintf(vflabel, 4, "J_%c", comp[jc]);
    t_zdf_grid_axis axis[1];
    memset(axis, 0, sizeof(axis));
    axis[0].min = 0.0;
    axis[0].max = current->box;
    axis[0].name = "x";
    axis[0].label = "x";
    axis[0].units = "c/\\omega_p";
    t_zdf_grid_info info;
    memset(&info, 0, sizeof(info));
    info.ndims = 1;
    info.name = vfname;
    info.label = vflabel;
    info.units = "e \\omega_p^2 / c";
    info.axis = axis;
    info.count[0] = current->nx;
    t_zdf_iteration iter = {.name = "ITERATION", .n = current->iter, .t = current->iter * current->dt,
                            .time_units = "1/\\omega_p"};
    zdf_save_grid(buf, zdf_float32, &info, &iter, "CURRENT");
    free(buf);
}

/* charge with one upper guard cell, folded unless the window moves
 * (spec_deposit_charge, particles.c:1093-1115) */
EXPORT void spec_deposit_charge(const t_species *spec, float *charge)
{
    spec_sync_host((t_species *)spec);
    const float q = spec->q;
    for (int i = 0; i < spec->np; i++) {
        const int idx = spec->part[i].ix;
        const float w1 = spec->part[i].x;
        charge[idx] += (1.0f - w1) * q;
        charge[idx + 1] += (w1)*q;
    }
    if (!spec->moving_window) charge[0] += charge[spec->nx];
}

/* axis quantity of particles i0 .. i0+np-1 (spec_pha_axis, particles.c:1272-1295) */
static void pha_axis(const t_species *spec, int i0, int np, int quant, float *axis)
{
    switch (quant) {
    case X1:
        for (int i = 0; i < np; i++) axis[i] = (spec->part[i0 + i].x + spec->part[i0 + i].ix) * spec->dx;
        break;
    case U1:
        for (int i = 0; i < np; i++) axis[i] = spec->part[i0 + i].ux;
        break;
    case U2:
        for (int i = 0; i < np; i++) axis[i] = spec->part[i0 + i].uy;
        break;
    case U3:
        for (int i = 0; i < np; i++) axis[i] = spec->part[i0 + i].uz;
        break;
    }
}

static const char *pha_axis_units(int quant)
{
    switch (quant) {
    case X1: return "c/\\omega_p";
    case U1:
    case U2:
    case U3: return "m_e c";
    }
    return "";
}

/* bilinear phase-space density (spec_deposit_pha, particles.c:1323-1390) */
EXPORT void spec_deposit_pha(const t_species *spec, const int rep_type, const int pha_nx[],
                             const float pha_range[][2], float *buf)
{
    spec_sync_host((t_species *)spec);
    enum { CHUNK = 1024 };
    float a1[CHUNK], a2[CHUNK];
    const int nrow = pha_nx[0];
    const int quant1 = rep_type & 0x000F;
    const int quant2 = (rep_type & 0x00F0) >> 4;
    const float x1min = pha_range[0][0];
    const float x2min = pha_range[1][0];
    const float rdx1 = pha_nx[0] / (pha_range[0][1] - pha_range[0][0]);
    const float rdx2 = pha_nx[1] / (pha_range[1][1] - pha_range[1][0]);
    for (int i = 0; i < spec->np; i += CHUNK) {
        const int np = (i + CHUNK > spec->np) ? spec->np - i : CHUNK;
        pha_axis(spec, i, np, quant1, a1);
        pha_axis(spec, i, np, quant2, a2);
        for (int k = 0; k < np; k++) {
            const float nx1 = (a1[k] - x1min) * rdx1;
            const float nx2 = (a2[k] - x2min) * rdx2;
            const int i1 = (int)(nx1 + 0.5f);
            const int i2 = (int)(nx2 + 0.5f);
            const float w1 = nx1 - i1 + 0.5f;
            const float w2 = nx2 - i2 + 0.5f;
            int idx = i1 + nrow * i2;
            if (i2 >= 0 && i2 < pha_nx[1]) {
                if (i1 >= 0 && i1 < pha_nx[0]) buf[idx] += (1.0f - w1) * (1.0f - w2) * spec->q;
                if (i1 + 1 >= 0 && i1 + 1 < pha_nx[0]) buf[idx + 1] += w1 * (1.0f - w2) * spec->q;
            }
            idx += nrow;
            if (i2 + 1 >= 0 && i2 + 1 < pha_nx[1]) {
                if (i1 >= 0 && i1 < pha_nx[0]) buf[idx] += (1.0f - w1) * w2 * spec->q;
                if (i1 + 1 >= 0 && i1 + 1 < pha_nx[0]) buf[idx + 1] += w1 * w2 * spec->q;
            }
        }
    }
}

static void rep_charge(const t_species *spec)
{
    float *charge = (float *)calloc((size_t)spec->nx + 1, sizeof(float));
    if (!charge) die("(*error*) out of memory");
    spec_deposit_charge(spec, charge);
    t_zdf_grid_axis axis;
    memset(&axis, 0, sizeof(axis));
    axis.min = spec->n_move * spec->dx;
    axis.max = spec->box + spec->n_move * spec->dx;
    axis.name = "x";
    axis.label = "x";
    axis.units = "c/\\omega_p";
    char name[128], label[128];
    snprintf(name, 128, "%s-charge", spec->name);
    snprintf(label, 128, "%s \\rho", spec->name);
    t_zdf_grid_info info;
    memset(&info, 0, sizeof(info));
    info.ndims = 1;
    info.name = name;
    info.label = label;
    info.units = "n_e";
    info.axis = &axis;
    info.count[0] = spec->nx;
    t_zdf_iteration iter = {.name = "ITERATION", .n = spec->iter, .t = spec->iter * spec->dt,
                            .time_units = "1/\\omega_p"};
    char path[1024];
    snprintf(path, 1024, "CHARGE/%s", spec->name);
    zdf_save_grid(charge, zdf_float32, &info, &iter, path);
    free(charge);
}

static void rep_pha(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2])
{
    float *buf = (float *)calloc((size_t)pha_nx[0] * pha_nx[1], sizeof(float));
    if (!buf) die("(*error*) out of memory");
    spec_deposit_pha(spec, rep_type, pha_nx, pha_range, buf);
    const int quant1 = rep_type & 0x000F;
    const int quant2 = (rep_type & 0x00F0) >> 4;
    const char *const ax_name[] = {"x1", "x2", "x3", "u1", "u2", "u3"};
    const char *const ax_label[] = {"x", "y", "z", "u_x", "u_y", "u_z"};
    t_zdf_grid_axis axis[2];
    memset(axis, 0, sizeof(axis));
    axis[0].min = pha_range[0][0];
    axis[0].max = pha_range[0][1];
    axis[0].name = (char *)ax_name[quant1 - 1];
    axis[0].label = (char *)ax_label[quant1 - 1];
    axis[0].units = (char *)pha_axis_units(quant1);
    axis[1].min = pha_range[1][0];
    axis[1].max = pha_range[1][1];
    axis[1].name = (char *)ax_name[quant2 - 1];
    axis[1].label = (char *)ax_label[quant2 - 1];
    axis[1].units = (char *)pha_axis_units(quant2);
    char pha_name[64], pha_label[64];
    snprintf(pha_name, 64, "%s-%s%s", spec->name, ax_name[quant1 - 1], ax_name[quant2 - 1]);
    snprintf(pha_label, 64, "%s %s-%s", spec->name, ax_label[quant1 - 1], ax_label[quant2 - 1]);
    t_zdf_grid_info info;
    memset(&info, 0, sizeof(info));
    info.ndims = 2;
    info.name = pha_name;
    info.label = pha_label;
    info.units = "a.u.";
    info.axis = axis;
    info.count[0] = pha_nx[0];
    info.count[1] = pha_nx[1];
    t_zdf_iteration iter = {.name = "ITERATION", .n = spec->iter, .t = spec->iter * spec->dt,
                            .time_units = "1/\\omega_p"};
    char path[1024];
    snprintf(path, 1024, "PHASESPACE/%s", spec->name);
    zdf_save_grid(buf, zdf_float32, &info, &iter, path);
    free(buf);
}

static void rep_particles(const t_species *spec)
{
    const char *quants[] = {"x", "ux", "uy", "uz"};
    const char *qlabels[] = {"x", "u_x", "u_y", "u_z"};
    const char *qunits[] = {"c/\\omega_p", "c", "c", "c"};
    t_zdf_iteration iter = {.name = "ITERATION", .n = spec->iter, .t = spec->iter * spec->dt,
                            .time_units = "1/\\omega_p"};
    t_zdf_part_info info;
    memset(&info, 0, sizeof(info));
    info.name = (char *)spec->name;
    info.label = (char *)spec->name;
    info.nquants = 4;
    info.quants = (char **)quants;
    info.qlabels = (char **)qlabels;
    info.qunits = (char **)qunits;
    info.np = spec->np;
    t_zdf_file part_file;
    char path[1024];
    snprintf(path, 1024, "PARTICLES/%s", spec->name);
    zdf_open_part_file(&part_file, &info, &iter, path);
    float *data = (float *)malloc(sizeof(float) * (size_t)(spec->np > 0 ? spec->np : 1));
    if (!data) die("(*error*) out of memory");
    for (int i = 0; i < spec->np; i++) data[i] = (spec->n_move + spec->part[i].ix + spec->part[i].x) * spec->dx;
    zdf_add_quant_part_file(&part_file, quants[0], data, spec->np);
    for (int i = 0; i < spec->np; i++) data[i] = spec->part[i].ux;
    zdf_add_quant_part_file(&part_file, quants[1], data, spec->np);
    for (int i = 0; i < spec->np; i++) data[i] = spec->part[i].uy;
    zdf_add_quant_part_file(&part_file, quants[2], data, spec->np);
    for (int i = 0; i < spec->np; i++) data[i] = spec->part[i].uz;
    zdf_add_quant_part_file(&part_file, quants[3], data, spec->np);
    free(data);
    zdf_close_file(&part_file);
}

EXPORT void spec_report(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2])
{
    spec_sync_host((t_species *)spec);
    switch (rep_type & 0xF000) {
    case CHARGE: rep_charge(spec); break;
    case PHA: rep_pha(spec, rep_type, pha_nx, pha_range); break;
    case PARTICLES: rep_particles(spec); break;
    }
}

/* ------------------------------------------------------------------------- */
/* timings and teardown                                                      */
/* ------------------------------------------------------------------------- */
static uint64_t live_npush(void)
{
    uint64_t n = g_npush;
    for (int k = 0; k < MAX_SIMS; k++) {
        entry_t *e = g_reg[k];
        if (!e || !e->gpu) continue;
        for (int s = 0; s < e->sim->n_species; s++) {
            long long v = 0;
            if (zc1_species_pushed(e->gpu, s, &v) == ZC_OK) n += (uint64_t)v;
        }
    }
    return n;
}

static double live_step_s(void)
{
    double t = g_step_s;
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k]) t += g_reg[k]->step_s;
    return t;
}

EXPORT uint64_t spec_npush(void) { return live_npush(); }
/* the whole GPU step: push and field advance run together */
EXPORT double spec_time(void) { return live_step_s(); }
EXPORT double emf_time(void) { return 0.0; }
EXPORT double spec_perf(void)
{
    const uint64_t n = live_npush();
    return (n > 0) ? live_step_s() / n : -1.0;
}

EXPORT void sim_timings(t_simulation *sim, uint64_t t0, uint64_t t1)
{
    entry_t *e = reg_by_sim(sim);
    if (e) gpu_wait(e);
    fprintf(stderr, "Time for spec. advance = %f s\n", spec_time());
    fprintf(stderr, "Time for emf   advance = %f s\n", emf_time());
    fprintf(stderr, "(the GPU step advances particles and fields together)\n");
    fprintf(stderr, "Total simulation time  = %f s\n", timer_interval_seconds(t0, t1));
    fprintf(stderr, "\n");
    const double perf = spec_perf();
    if (perf > 0) {
        fprintf(stderr, "Particle advance [nsec/part] = %f \n", 1.e9 * perf);
        fprintf(stderr, "Particle advance [Mpart/sec] = %f \n", 1.e-6 / perf);
    }
}

EXPORT void sim_delete(t_simulation *sim)
{
    entry_t *e = reg_by_sim(sim);
    if (e && e->gpu) {
        gpu_wait(e);
        for (int k = 0; k < sim->n_species; k++) {
            long long v = 0;
            if (zc1_species_pushed(e->gpu, k, &v) == ZC_OK) g_npush += (uint64_t)v;
        }
        g_step_s += e->step_s;
        zc1_destroy(e->gpu);
        e->gpu = NULL;
    }
    zdf_flush();
    for (int i = 0; i < sim->n_species; i++) spec_delete(&sim->species[i]);
    free(sim->species);
    sim->species = NULL;
    current_delete(&sim->current);
    emf_delete(&sim->emf);
    if (e) reg_remove(e);
}
