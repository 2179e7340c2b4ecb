/*
 * em2d_host.c -- libzpic_em2d: ZPIC's em2d C API (include/em2d/*.h) on top
 * of the libzpic_cuda C-ABI.
 *
 * What runs here, on the host, in plain C99:
 *   - the process-global MWC generator and polar Box-Muller deviates
 *     (reference em2d/random.c:16-101), so that particle loading draws the
 *     same numbers in the same order as the reference;
 *   - particle loading and moving-window injection (spec_new and its helpers,
 *     reference em2d/particles.c:85-612) into host buffers in the reference
 *     record layout, handed to the GPU through zc_species_create /
 *     the injection provider;
 *   - parameter checks with the reference's exit(-1) behaviour
 *     (em2d/simulation.c:106-110, 136-146; em2d/emf.c:246-270);
 *   - host mirrors of the device state (t_species.part, t_emf.E_buf/B_buf,
 *     t_current.J_buf), kept valid across every sim_iter (edits uploaded
 *     before the step, all mirrors refreshed after it) unless
 *     ZPIC_EM2D_MIRRORS=demand, in which case sim_sync_host and the reports
 *     refresh them;
 *   - the ZDF report files, gathered from the device and written on a
 *     background thread (zdf_io.c).
 * Everything per time step (push, deposit, current update, field advance,
 * moving window) runs on the GPU via zc_step / the zc_* phase calls.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>

#include <pthread.h>

#include "../../../include/em2d/simulation.h"
#include "../../../include/em2d/zdf.h"
#include "../../../include/em2d/random.h"
#include "../../../include/em2d/timer.h"
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
/* host passes over the mirrors (compare, copy), split over host threads:    */
/* a 2048 x 2048 grid at 16 particles per cell keeps 1.9 GB of particle      */
/* mirrors, which one thread compares or copies in about 0.1 s               */
/* ------------------------------------------------------------------------- */
typedef struct {
    const unsigned char *src;
    const unsigned char *cmp;  /* compare: the other span */
    unsigned char *dst;        /* copy: the destination */
    size_t n;
    int differ;
} span_job;

static void *span_run(void *arg)
{
    span_job *j = (span_job *)arg;
    if (j->dst) memcpy(j->dst, j->src, j->n);
    else j->differ = j->n > 0 && memcmp(j->cmp, j->src, j->n) != 0;
    return NULL;
}

static int host_threads(void)
{
    static int n = 0;
    if (!n) {
        const long c = sysconf(_SC_NPROCESSORS_ONLN);
        n = c < 1 ? 1 : (c > 16 ? 16 : (int)c);
    }
    return n;
}

/* dst != NULL: copies src to dst; else compares src with cmp and returns
 * nonzero if they differ.  Spans of at least 4 MB, one thread each. */
static int span_pass(unsigned char *dst, const unsigned char *cmp, const unsigned char *src, size_t n)
{
    enum { MAXT = 16 };
    int nt = (int)(n / ((size_t)4 << 20));
    if (nt > host_threads()) nt = host_threads();
    if (nt < 1) nt = 1;
    span_job job[MAXT];
    pthread_t th[MAXT];
    int started[MAXT];
    const size_t step = (n + (size_t)nt - 1) / (size_t)nt;
    for (int t = 0; t < nt; t++) {
        const size_t a = (size_t)t * step < n ? (size_t)t * step : n;
        const size_t b = a + step < n ? a + step : n;
        job[t].src = src + a;
        job[t].cmp = cmp ? cmp + a : NULL;
        job[t].dst = dst ? dst + a : NULL;
        job[t].n = b - a;
        job[t].differ = 0;
        started[t] = 0;
    }
    for (int t = 1; t < nt; t++) started[t] = pthread_create(&th[t], NULL, span_run, &job[t]) == 0;
    span_run(&job[0]);
    int differ = job[0].differ;
    for (int t = 1; t < nt; t++) {
        if (started[t]) pthread_join(th[t], NULL);
        else span_run(&job[t]);
        differ |= job[t].differ;
    }
    return differ;
}

static int mirror_differs(const void *a, const void *b, size_t n)
{
    return span_pass(NULL, (const unsigned char *)a, (const unsigned char *)b, n);
}

static void mirror_copy(void *dst, const void *src, size_t n)
{
    span_pass((unsigned char *)dst, NULL, (const unsigned char *)src, n);
}

/* ------------------------------------------------------------------------- */
/* timers (reference em2d/timer.c)                                           */
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
/* random numbers: multiply-with-carry pair (Marsaglia) + polar Box-Muller   */
/* ------------------------------------------------------------------------- */
/* One generator per host thread: a single-threaded program sees the
 * reference's process-global generator (random.c:16-17); threads that load
 * different runs of a scan at once do not share (or race on) one state. */
static __thread uint32_t g_w = 12345, g_z = 67890;   /* the reference's default seeds */
static __thread int g_spare_ok = 0;
static __thread double g_spare = 0.0;

EXPORT void set_rand_seed(uint32_t w, uint32_t z)
{
    /* the cached deviate is kept, as in the reference */
    g_w = w;
    g_z = z;
}

/* No counterpart in the reference: seeds the generator and drops the cached
 * deviate, i.e. the state of a newly started process after set_rand_seed.
 * A scan that loads each run this way gives every run the particles it gets
 * as a process of its own, whatever order the runs are loaded in. */
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
/* registry: C structs of a simulation -> its GPU handle                     */
/* ------------------------------------------------------------------------- */
typedef struct {
    t_simulation *sim;
    zc_sim *gpu;
    zc_part *inj;      /* injection buffer, owned here */
    int inj_cap;
    /* host mirrors kept valid across sim_iter (see mirrors_mode): the state
     * of every mirror as last synchronised, to find edits made in between */
    int mirrors;
    t_part **shadow;
    int *shadow_np, *shadow_cap;
    float3 *shadow_E, *shadow_B;
} entry_t;

#define MAX_SIMS 4096
static entry_t g_reg[MAX_SIMS];

static entry_t *reg_add(t_simulation *sim)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (!g_reg[k].sim) {
            memset(&g_reg[k], 0, sizeof(entry_t));
            g_reg[k].sim = sim;
            return &g_reg[k];
        }
    die("(*error*) too many simulations");
    return NULL;
}

static entry_t *reg_by_sim(const t_simulation *sim)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k].sim == sim) return &g_reg[k];
    return NULL;
}

static entry_t *reg_by_emf(const t_emf *emf)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k].sim && &g_reg[k].sim->emf == emf) return &g_reg[k];
    return NULL;
}

static entry_t *reg_by_current(const t_current *cur)
{
    for (int k = 0; k < MAX_SIMS; k++)
        if (g_reg[k].sim && &g_reg[k].sim->current == cur) return &g_reg[k];
    return NULL;
}

static entry_t *reg_by_species(const t_species *sp, int *index)
{
    for (int k = 0; k < MAX_SIMS; k++) {
        t_simulation *s = g_reg[k].sim;
        if (s && sp >= s->species && sp < s->species + s->n_species) {
            *index = (int)(sp - s->species);
            return &g_reg[k];
        }
    }
    return NULL;
}

static entry_t *need(entry_t *e, const char *where)
{
    if (!e) {
        fprintf(stderr, "(*error*) %s: object is not part of a simulation created by sim_new\n", where);
        exit(-1);
    }
    return e;
}

/* options for the next sim_new */
static int g_device = 0, g_tile[2] = {16, 16}, g_fast = 0;

EXPORT void sim_set_gpu_options(int device, int tile_x, int tile_y, int fast_math)
{
    g_device = device;
    g_tile[0] = tile_x > 0 ? tile_x : 16;
    g_tile[1] = tile_y > 0 ? tile_y : 16;
    g_fast = fast_math ? 1 : 0;
}

/* ------------------------------------------------------------------------- */
/* particle loading (reference em2d/particles.c:85-612)                      */
/* ------------------------------------------------------------------------- */
static float unit_profile(float x, void *d)
{
    (void)x;
    (void)d;
    return 1.0f;
}

EXPORT void spec_grow_buffer(t_species *spec, const int size)
{
    if (size > spec->np_max) {
        spec->np_max = (size / 1024 + 1) * 1024;
        t_part *p = (t_part *)realloc(spec->part, (size_t)spec->np_max * sizeof(t_part));
        if (!p) die("(*error*) unable to grow particle buffer");
        spec->part = p;
    }
}

/* momenta of particles first..last: thermal draw, per-cell mean removed,
 * fluid drift added (particles.c:85-149) */
static void load_momenta(t_species *sp, int first, int last)
{
    for (int k = first; k <= last; k++) {
        sp->part[k].ux = sp->uth[0] * rand_norm();
        sp->part[k].uy = sp->uth[1] * rand_norm();
        sp->part[k].uz = sp->uth[2] * rand_norm();
    }
    /* The per-cell table is indexed with stride nx[1], as the reference
     * indexes its table of nx[0]*nx[1] entries (particles.c:104-105,116).
     * With nx[1] > nx[0] the reference's indices run past its table
     * (undefined behaviour); here the table holds every index and all its
     * entries are normalised, so each cell's mean is removed.  With
     * nx[1] <= nx[0] the arithmetic is the reference's exactly. */
    const int stride = sp->nx[1];
    const int ncell = sp->nx[0] * sp->nx[1];
    const int nidx = (sp->nx[0] - 1) + stride * (sp->nx[1] - 1) + 1;
    const int ntab = nidx > ncell ? nidx : ncell;
    float3 *mean = (float3 *)calloc((size_t)ntab, sizeof(float3));
    int *cnt = (int *)calloc((size_t)ntab, sizeof(int));
    if (!mean || !cnt) die("(*error*) out of memory");
    for (int k = first; k <= last; k++) {
        const int c = sp->part[k].ix + stride * sp->part[k].iy;
        mean[c].x += sp->part[k].ux;
        mean[c].y += sp->part[k].uy;
        mean[c].z += sp->part[k].uz;
        cnt[c] += 1;
    }
    for (int c = 0; c < ntab; c++) {
        const float w = (cnt[c] > 0) ? 1.0f / cnt[c] : 0;
        mean[c].x *= w;
        mean[c].y *= w;
        mean[c].z *= w;
    }
    for (int k = first; k <= last; k++) {
        const int c = sp->part[k].ix + stride * sp->part[k].iy;
        sp->part[k].ux += sp->ufl[0] - mean[c].x;
        sp->part[k].uy += sp->ufl[1] - mean[c].y;
        sp->part[k].uz += sp->ufl[2] - mean[c].z;
    }
    free(cnt);
    free(mean);
}

/* upper bound of the particles placed in a cell range (particles.c:367-449) */
static int count_for_range(t_species *sp, const int r[2][2])
{
    int n = 0;
    switch (sp->density.type) {
    case STEP: {
        int i0 = sp->density.start / sp->dx[0] - sp->n_move;
        if (i0 > r[0][1]) n = 0;
        else {
            if (i0 < r[0][0]) i0 = r[0][0];
            n = (r[0][1] - i0 + 1) * sp->ppc[0];
        }
        n *= (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    } break;
    case SLAB: {
        int i0 = sp->density.start / sp->dx[0] - sp->n_move;
        int i1 = sp->density.end / sp->dx[1] - sp->n_move;  /* dx[1], as the reference */
        if (i0 > r[0][1] || i1 < r[0][0]) n = 0;
        else {
            if (i0 < r[0][0]) i0 = r[0][0];
            if (i1 > r[0][1]) i1 = r[0][1];
            n = (i1 - i0 + 1) * sp->ppc[0];
        }
        n *= (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    } break;
    case CUSTOM: {
        double x = (r[0][0] + sp->n_move) * sp->dx[0];
        double qx = sp->density.custom_x(x, sp->density.custom_data_x);
        x = (r[0][1] + 1 + sp->n_move) * sp->dx[0];
        qx += sp->density.custom_x(x, sp->density.custom_data_x);
        qx *= 0.5;
        for (int i = r[0][0] + 1; i <= r[0][1]; i++) {
            x = (i + sp->n_move) * sp->dx[0];
            qx += sp->density.custom_x(x, sp->density.custom_data_x);
        }
        double y = r[1][0] * sp->dx[1];
        double qy = sp->density.custom_y(y, sp->density.custom_data_y);
        y = (r[1][1] + 1) * sp->dx[1];
        qy += sp->density.custom_y(y, sp->density.custom_data_y);
        qy *= 0.5;
        for (int j = r[1][0] + 1; j <= r[1][1]; j++) {
            y = j * sp->dx[1];
            qy += sp->density.custom_y(y, sp->density.custom_data_y);
        }
        n = ceil(qx * sp->ppc[0]) * ceil(qy * sp->ppc[1]);
    } break;
    case EMPTY:
        n = 0;
        break;
    default:
        n = (r[0][1] - r[0][0] + 1) * sp->ppc[0] * (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    }
    return n;
}

static void put(t_species *sp, int *n, int i, int j, float x, float y)
{
    sp->part[*n].ix = i;
    sp->part[*n].iy = j;
    sp->part[*n].x = x;
    sp->part[*n].y = y;
    (*n)++;
}

/* positions from the density profile (particles.c:159-354) */
static void place(t_species *sp, const int r[2][2])
{
    const int npc = sp->ppc[0] * sp->ppc[1];
    const float hx = 1.0f / sp->ppc[0], hy = 1.0f / sp->ppc[1];
    float *lat = (float *)malloc(2 * (size_t)npc * sizeof(float));
    if (!lat) die("(*error*) out of memory");
    for (int b = 0, m = 0; b < sp->ppc[1]; b++)
        for (int a = 0; a < sp->ppc[0]; a++, m += 2) {
            lat[m] = hx * (a + 0.5);
            lat[m + 1] = hy * (b + 0.5);
        }
    int n = sp->np;
    if (sp->density.type == STEP || sp->density.type == SLAB) {
        const float lo = sp->density.start / sp->dx[0] - sp->n_move;
        const float hi = sp->density.end / sp->dx[0] - sp->n_move;
        const int slab = sp->density.type == SLAB;
        for (int j = r[1][0]; j <= r[1][1]; j++)
            for (int i = r[0][0]; i <= r[0][1]; i++)
                for (int k = 0; k < npc; k++) {
                    const float xp = i + lat[2 * k];
                    if (xp > lo && (!slab || xp < hi)) put(sp, &n, i, j, lat[2 * k], lat[2 * k + 1]);
                }
    } else if (sp->density.type == CUSTOM) {
        /* inverse cumulative distribution of the piecewise-linear profile,
         * continued across injections through the running totals */
        const double ddx = sp->dx[0], ddy = sp->dx[1];
        const double wx = 1.0 / sp->ppc[0], wy = 1.0 / sp->ppc[1];
        const double floor_n = 4 * wx * wy;
        const int mv = sp->n_move, i0 = r[0][0], j0 = r[1][0];
        unsigned long kx = sp->density.custom_x_total_part;
        double cx_hi = sp->density.custom_x_total_q, cx_lo;
        double nx_lo, nx_hi = sp->density.custom_x((i0 + mv) * ddx, sp->density.custom_data_x);
        const double ny_start = sp->density.custom_y(j0 * ddy, sp->density.custom_data_y);
        for (int i = i0; i <= r[0][1]; i++) {
            nx_lo = nx_hi;
            nx_hi = sp->density.custom_x((i + 1 + mv) * ddx, sp->density.custom_data_x);
            cx_lo = cx_hi;
            cx_hi += 0.5 * (nx_lo + nx_hi);
            double tx;
            while ((tx = (kx + 0.5) * wx) < cx_hi) {
                const double px = 2 * (tx - cx_lo) / (sqrt(nx_lo * nx_lo + 2 * (nx_hi - nx_lo) * (tx - cx_lo)) + nx_lo);
                const double dens_x = (0.5 - px) * nx_lo + (0.5 + px) * nx_hi;
                unsigned long ky = 0;
                double ny_lo, ny_hi = ny_start, cy_lo, cy_hi = 0;
                for (int j = j0; j <= r[1][1]; j++) {
                    ny_lo = ny_hi;
                    ny_hi = sp->density.custom_y((j + 1) * ddy, sp->density.custom_data_y);
                    cy_lo = cy_hi;
                    cy_hi += 0.5 * (ny_lo + ny_hi);
                    double ty;
                    while ((ty = (ky + 0.5) * wy) < cy_hi) {
                        const double py = 2 * (ty - cy_lo) / (sqrt(ny_lo * ny_lo + 2 * (ny_hi - ny_lo) * (ty - cy_lo)) + ny_lo);
                        const double dens_y = (0.5 - py) * ny_lo + (0.5 + py) * ny_hi;
                        if (dens_x * dens_y > floor_n) put(sp, &n, i, j, px, py);
                        ky++;
                    }
                }
                kx++;
            }
        }
        sp->density.custom_x_total_q = cx_hi;
        sp->density.custom_x_total_part = kx;
    } else if (sp->density.type != EMPTY) {
        for (int j = r[1][0]; j <= r[1][1]; j++)
            for (int i = r[0][0]; i <= r[0][1]; i++)
                for (int k = 0; k < npc; k++) put(sp, &n, i, j, lat[2 * k], lat[2 * k + 1]);
    }
    sp->np = n;
    free(lat);
}

static void inject(t_species *sp, const int r[2][2])  /* particles.c:476-492 */
{
    const int first = sp->np;
    spec_grow_buffer(sp, sp->np + count_for_range(sp, r));
    place(sp, r);
    load_momenta(sp, first, sp->np - 1);
}

EXPORT void spec_new(t_species *spec, char name[], const float m_q, const int ppc[], const float *ufl,
                     const float *uth, const int nx[], float box[], const float dt, t_density *density)
{
    strncpy(spec->name, name ? name : "", MAX_SPNAME_LEN);
    spec->name[MAX_SPNAME_LEN] = 0;
    int npc = 1;
    for (int d = 0; d < 2; d++) {
        spec->nx[d] = nx[d];
        spec->ppc[d] = ppc[d];
        npc *= ppc[d];
        spec->box[d] = box[d];
        spec->dx[d] = box[d] / nx[d];
    }
    spec->m_q = m_q;
    spec->q = copysignf(1.0f, m_q) / npc;
    spec->dt = dt;
    spec->np_max = 0;
    spec->part = NULL;
    if (density) spec->density = *density;
    else {
        memset(&spec->density, 0, sizeof(spec->density));
        spec->density.type = UNIFORM;
        spec->density.n = 1.0;
    }
    if (spec->density.n == 0.) spec->density.n = 1.0;
    if (spec->density.type == CUSTOM) {
        if (!spec->density.custom_x) spec->density.custom_x = unit_profile;
        if (!spec->density.custom_y) spec->density.custom_y = unit_profile;
        spec->density.custom_x_total_part = 0;
        spec->density.custom_x_total_q = 0;
    }
    spec->q *= fabsf(spec->density.n);
    for (int d = 0; d < 3; d++) {
        spec->ufl[d] = ufl ? ufl[d] : 0;
        spec->uth[d] = uth ? uth[d] : 0;
    }
    spec->energy = 0;
    spec->iter = 0;
    spec->moving_window = 0;
    spec->n_move = 0;
    spec->np = 0;
    const int r[2][2] = {{0, nx[0] - 1}, {0, nx[1] - 1}};
    inject(spec, r);
    spec->n_sort = 16;
}

EXPORT void spec_delete(t_species *spec)
{
    free(spec->part);
    spec->part = NULL;
    spec->np = -1;
}

/* moving-window injection provider for the GPU: the particles of the new
 * right-most column, drawn exactly as spec_move_window does
 * (particles.c:619-640); the shift of the existing particles is done on the
 * GPU */
static int provide_column(void *user, int k, int n_move, const zc_part **parts, int *np)
{
    entry_t *e = (entry_t *)user;
    t_species *sp = &e->sim->species[k];
    t_species tmp = *sp;
    tmp.part = (t_part *)e->inj;
    tmp.np_max = e->inj_cap;
    tmp.np = 0;
    tmp.n_move = n_move;
    const int r[2][2] = {{sp->nx[0] - 1, sp->nx[0] - 1}, {0, sp->nx[1] - 1}};
    inject(&tmp, r);
    e->inj = (zc_part *)tmp.part;  /* may have grown */
    e->inj_cap = tmp.np_max;
    sp->n_move = n_move;
    sp->density.custom_x_total_part = tmp.density.custom_x_total_part;
    sp->density.custom_x_total_q = tmp.density.custom_x_total_q;
    *parts = e->inj;
    *np = tmp.np;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* fields and current: host mirrors (reference em2d/emf.c:56-115,            */
/* em2d/current.c:30-79)                                                     */
/* ------------------------------------------------------------------------- */
EXPORT void emf_new(t_emf *emf, int nx[], float box[], const float dt)
{
    memset(emf, 0, sizeof(*emf));
    for (int d = 0; d < 2; d++) {
        emf->nx[d] = nx[d];
        emf->gc[d][0] = 1;
        emf->gc[d][1] = 2;
        emf->box[d] = box[d];
        emf->dx[d] = box[d] / nx[d];
    }
    emf->nrow = nx[0] + 3;
    const size_t n = (size_t)(nx[0] + 3) * (nx[1] + 3);
    emf->E_buf = (float3 *)calloc(n, sizeof(float3));
    emf->B_buf = (float3 *)calloc(n, sizeof(float3));
    if (!emf->E_buf || !emf->B_buf) die("(*error*) out of memory");
    emf->E = emf->E_buf + 1 + emf->nrow;
    emf->B = emf->B_buf + 1 + emf->nrow;
    emf->E_part = emf->E;
    emf->B_part = emf->B;
    emf->dt = dt;
}

EXPORT void emf_delete(t_emf *emf)
{
    free(emf->E_buf);
    free(emf->B_buf);
    free(emf->ext_fld.E_part_buf);
    free(emf->ext_fld.B_part_buf);
    emf->E_buf = emf->B_buf = NULL;
    emf->ext_fld.E_part_buf = emf->ext_fld.B_part_buf = NULL;
    emf->E_part = emf->B_part = NULL;
}

EXPORT void current_new(t_current *current, int nx[], float box[], float dt)
{
    memset(current, 0, sizeof(*current));
    for (int d = 0; d < 2; d++) {
        current->nx[d] = nx[d];
        current->gc[d][0] = 1;
        current->gc[d][1] = 2;
        current->box[d] = box[d];
        current->dx[d] = box[d] / nx[d];
    }
    current->nrow = nx[0] + 3;
    current->J_buf = (float3 *)calloc((size_t)(nx[0] + 3) * (nx[1] + 3), sizeof(float3));
    if (!current->J_buf) die("(*error*) out of memory");
    current->J = current->J_buf + 1 + current->nrow;
    current->dt = dt;
}

EXPORT void current_delete(t_current *current)
{
    free(current->J_buf);
    current->J_buf = NULL;
}

/* ------------------------------------------------------------------------- */
/* simulation (reference em2d/simulation.c)                                  */
/* ------------------------------------------------------------------------- */
static double g_spec_time = 0, g_emf_time = 0;
static uint64_t g_npush = 0;

EXPORT uint64_t spec_npush(void) { return g_npush; }
EXPORT double spec_time(void) { return g_spec_time; }
EXPORT double spec_perf(void) { return (g_npush > 0) ? g_spec_time / g_npush : -1.0; }
EXPORT double emf_time(void) { return g_emf_time; }

EXPORT int report(int n, int ndump) { return (ndump > 0) ? !(n % ndump) : 0; }

/* Mirror policy of a new simulation.  The reference's structs are read and
 * written directly by its callers (the Cython module's Species.particles,
 * EMF.Ex ... views, em2d.pyx:306-312,1055-1060; decks that read
 * species->part in sim_report).  By default every sim_iter therefore uploads
 * what was edited in the mirrors since the last step (particles, E, B) and
 * refreshes every mirror after the step, so direct reads and writes behave
 * as with the reference.  ZPIC_EM2D_MIRRORS=demand turns that off: the
 * mirrors are then refreshed only by sim_sync_host and the reports, and
 * edits are uploaded only by sim_sync_device (no per-step copies). */
static int mirrors_mode(void)
{
    const char *v = getenv("ZPIC_EM2D_MIRRORS");
    return !(v && strcmp(v, "demand") == 0);
}

static void shadow_save(entry_t *e);
static void refresh_mirrors(entry_t *e);

EXPORT void sim_new(t_simulation *sim, int nx[], float box[], float dt, float tmax, int ndump,
                    t_species *species, int n_species)
{
    sim->dt = dt;
    sim->tmax = tmax;
    sim->ndump = ndump;
    emf_new(&sim->emf, nx, box, dt);
    current_new(&sim->current, nx, box, dt);
    sim->n_species = n_species;
    sim->species = species;
    sim->moving_window = 0;
    const float cour = sqrtf(1.0f / (1.0f / (sim->emf.dx[0] * sim->emf.dx[0]) +
                                     1.0f / (sim->emf.dx[1] * sim->emf.dx[1])));
    if (dt >= cour) {
        fprintf(stderr, "Invalid timestep, courant condition violation, dtmax = %f \n", cour);
        exit(-1);
    }
    entry_t *e = reg_add(sim);
    zc_sim_desc d;
    memset(&d, 0, sizeof(d));
    d.nx[0] = nx[0];
    d.nx[1] = nx[1];
    d.box[0] = box[0];
    d.box[1] = box[1];
    d.dt = dt;
    d.device = g_device;
    d.tile[0] = g_tile[0];
    d.tile[1] = g_tile[1];
    d.fast_math = g_fast;
    zc_check(zc_sim_create(&d, &e->gpu), "sim_new");
    for (int k = 0; k < n_species; k++) {
        zc_species_desc sd;
        sd.m_q = species[k].m_q;
        sd.q = species[k].q;
        sd.ppc[0] = species[k].ppc[0];
        sd.ppc[1] = species[k].ppc[1];
        int id;
        zc_check(zc_species_create(e->gpu, &sd, (const zc_part *)species[k].part, species[k].np, &id),
                 "sim_new (species upload)");
    }
    zc_check(zc_set_injector(e->gpu, provide_column, e), "sim_new");
    e->mirrors = mirrors_mode();
    if (e->mirrors) shadow_save(e);
}

EXPORT void sim_delete(t_simulation *sim)
{
    zdf_flush();  /* report files still queued may wait on this simulation's copies */
    entry_t *e = reg_by_sim(sim);
    if (e) {
        zc_sim_destroy(e->gpu);
        free(e->inj);
        if (e->shadow)
            for (int k = 0; k < sim->n_species; k++) free(e->shadow[k]);
        free(e->shadow);
        free(e->shadow_np);
        free(e->shadow_cap);
        free(e->shadow_E);
        free(e->shadow_B);
        memset(e, 0, sizeof(*e));
    }
    for (int k = 0; k < sim->n_species; k++) spec_delete(&sim->species[k]);
    free(sim->species);
    current_delete(&sim->current);
    emf_delete(&sim->emf);
}

/* bookkeeping after n device steps: the counters the reference keeps on the
 * host structs, and the timing totals of sim_timings (the push count uses
 * the particle count of the last host sync, which is exact unless a moving
 * window adds or removes particles) */
static void after_steps(entry_t *e, int nsteps, int species_only, int k_only)
{
    t_simulation *sim = e->sim;
    float ms = 0;
    zc_last_step_ms(e->gpu, &ms);
    for (int k = 0; k < sim->n_species; k++) {
        if (species_only && k != k_only) continue;
        sim->species[k].iter += nsteps;
        g_npush += (uint64_t)(sim->species[k].np > 0 ? sim->species[k].np : 0) * nsteps;
    }
    if (!species_only) {
        sim->current.iter += nsteps;
        sim->emf.iter += nsteps;
        zc_info info;
        zc_get_info(e->gpu, &info);
        sim->emf.n_move = info.n_move;
    }
    g_spec_time += ms * 1e-3;
}

static void push_host_edits(entry_t *e);

EXPORT void sim_iter(t_simulation *sim)
{
    entry_t *e = need(reg_by_sim(sim), "sim_iter");
    if (e->mirrors) push_host_edits(e);
    zc_check(zc_step(e->gpu, 1), "sim_iter");
    after_steps(e, 1, 0, 0);
    if (e->mirrors) refresh_mirrors(e);
}

EXPORT void spec_advance(t_species *spec, t_emf *emf, t_current *current)
{
    (void)current;
    int k = 0;
    entry_t *e = need(reg_by_species(spec, &k), "spec_advance");
    if (reg_by_emf(emf) != e) need(NULL, "spec_advance (fields of another simulation)");
    zc_check(zc_spec_advance(e->gpu, k), "spec_advance");
    after_steps(e, 1, 1, k);
}

EXPORT void current_zero(t_current *current)
{
    entry_t *e = reg_by_current(current);
    if (!e) {  /* a stand-alone current object: plain host buffer */
        memset(current->J_buf, 0, (size_t)(current->nx[0] + 3) * (current->nx[1] + 3) * sizeof(float3));
        return;
    }
    zc_check(zc_current_zero(e->gpu), "current_zero");
}

EXPORT void current_update(t_current *current)
{
    entry_t *e = need(reg_by_current(current), "current_update");
    zc_check(zc_current_update(e->gpu), "current_update");
    current->iter++;
}

EXPORT void emf_advance(t_emf *emf, const t_current *current)
{
    (void)current;
    entry_t *e = need(reg_by_emf(emf), "emf_advance");
    const uint64_t t0 = timer_ticks();
    zc_check(zc_emf_advance(e->gpu), "emf_advance");
    emf->iter++;
    zc_info info;
    zc_get_info(e->gpu, &info);
    emf->n_move = info.n_move;
    g_emf_time += timer_interval_seconds(t0, timer_ticks());
}

EXPORT void sim_timings(t_simulation *sim, uint64_t t0, uint64_t t1)
{
    (void)sim;
    fprintf(stderr, "Time for spec. advance = %f s\n", spec_time());
    fprintf(stderr, "Time for emf   advance = %f s\n", emf_time());
    fprintf(stderr, "Total simulation time  = %f s\n", timer_interval_seconds(t0, t1));
    fprintf(stderr, "\n");
    const double perf = spec_perf();
    if (perf > 0) {
        fprintf(stderr, "Particle advance [nsec/part] = %f \n", 1.e9 * perf);
        fprintf(stderr, "Particle advance [Mpart/sec] = %f \n", 1.e-6 / perf);
    }
}

EXPORT void sim_add_laser(t_simulation *sim, t_emf_laser *laser) { emf_add_laser(&sim->emf, laser); }

EXPORT void emf_add_laser(t_emf *const emf, t_emf_laser *laser)
{
    entry_t *e = need(reg_by_emf(emf), "emf_add_laser");
    /* parameter checks and exit codes of the reference (emf.c:245-270) */
    if (laser->fwhm != 0) {
        if (laser->fwhm <= 0) die("Invalid laser FWHM, must be > 0, aborting.");
        laser->rise = laser->fwhm;
        laser->fall = laser->fwhm;
        laser->flat = 0.;
    }
    if (laser->rise <= 0) die("Invalid laser RISE, must be > 0, aborting.");
    if (laser->flat < 0) die("Invalid laser FLAT, must be >= 0, aborting.");
    if (laser->fall <= 0) die("Invalid laser FALL, must be > 0, aborting.");
    zc_laser L;
    L.type = laser->type;
    L.start = laser->start;
    L.fwhm = laser->fwhm;
    L.rise = laser->rise;
    L.flat = laser->flat;
    L.fall = laser->fall;
    L.a0 = laser->a0;
    L.omega0 = laser->omega0;
    L.polarization = laser->polarization;
    L.W0 = laser->W0;
    L.focus = laser->focus;
    L.axis = laser->axis;
    zc_check(zc_add_laser(e->gpu, &L), "emf_add_laser");
    if (e->mirrors) refresh_mirrors(e);
}

EXPORT void sim_set_smooth(t_simulation *sim, t_smooth *smooth)
{
    if (smooth->xtype != NONE && smooth->xlevel <= 0) die("Invalid smooth level along x direction");
    if (smooth->ytype != NONE && smooth->ylevel <= 0) die("Invalid smooth level along y direction");
    sim->current.smooth = *smooth;
    entry_t *e = need(reg_by_sim(sim), "sim_set_smooth");
    zc_check(zc_set_smooth(e->gpu, smooth->xtype, smooth->xlevel, smooth->ytype, smooth->ylevel),
             "sim_set_smooth");
}

EXPORT void sim_set_moving_window(t_simulation *sim)
{
    entry_t *e = need(reg_by_sim(sim), "sim_set_moving_window");
    sim->emf.moving_window = 1;
    sim->current.moving_window = 1;
    for (int k = 0; k < sim->n_species; k++) sim->species[k].moving_window = 1;
    zc_check(zc_set_moving_window(e->gpu), "sim_set_moving_window");
}

/* evaluates a custom field callback over every buffer cell, reference
 * layout (the same cells emf_update_part_fld / emf_init_fld visit) */
static float3 *eval_grid(const t_emf *emf, float3 (*fn)(int, float, int, float, void *), void *data)
{
    const int nrow = emf->nrow;
    float3 *g = (float3 *)calloc((size_t)nrow * (emf->nx[1] + 3), sizeof(float3));
    if (!g) die("(*error*) out of memory");
    for (int j = -1; j < emf->nx[1] + 2; j++)
        for (int i = -1; i < emf->nx[0] + 2; i++) g[(j + 1) * nrow + i + 1] = fn(i, emf->dx[0], j, emf->dx[1], data);
    return g;
}

EXPORT void sim_set_ext_fld(t_simulation *sim, t_emf_ext_fld *ext_fld) { emf_set_ext_fld(&sim->emf, ext_fld); }

EXPORT void emf_set_ext_fld(t_emf *const emf, t_emf_ext_fld *ext)
{
    entry_t *e = need(reg_by_emf(emf), "emf_set_ext_fld");
    if (ext->E_type > EMF_FLD_TYPE_CUSTOM || ext->B_type > EMF_FLD_TYPE_CUSTOM)
        die("Invalid external field type, aborting.");
    float E0[3] = {ext->E_0.x, ext->E_0.y, ext->E_0.z}, B0[3] = {ext->B_0.x, ext->B_0.y, ext->B_0.z};
    float3 *Eg = NULL, *Bg = NULL;
    if (ext->E_type == EMF_FLD_TYPE_CUSTOM) Eg = eval_grid(emf, ext->E_custom, ext->E_custom_data);
    if (ext->B_type == EMF_FLD_TYPE_CUSTOM) Bg = eval_grid(emf, ext->B_custom, ext->B_custom_data);
    emf->ext_fld.E_type = ext->E_type;
    emf->ext_fld.B_type = ext->B_type;
    emf->ext_fld.E_0 = ext->E_0;
    emf->ext_fld.B_0 = ext->B_0;
    emf->ext_fld.E_custom = ext->E_custom;
    emf->ext_fld.B_custom = ext->B_custom;
    emf->ext_fld.E_custom_data = ext->E_custom_data;
    emf->ext_fld.B_custom_data = ext->B_custom_data;
    zc_check(zc_set_ext_fld(e->gpu, ext->E_type, E0, (const float *)Eg, ext->B_type, B0, (const float *)Bg),
             "emf_set_ext_fld");
    free(Eg);
    free(Bg);
    /* host mirrors of the particle fields */
    const size_t n = (size_t)emf->nrow * (emf->nx[1] + 3);
    if (ext->E_type != EMF_FLD_TYPE_NONE) {
        if (!emf->ext_fld.E_part_buf) emf->ext_fld.E_part_buf = (float3 *)calloc(n, sizeof(float3));
        emf->E_part = emf->ext_fld.E_part_buf + 1 + emf->nrow;
    } else emf->E_part = emf->E;
    if (ext->B_type != EMF_FLD_TYPE_NONE) {
        if (!emf->ext_fld.B_part_buf) emf->ext_fld.B_part_buf = (float3 *)calloc(n, sizeof(float3));
        emf->B_part = emf->ext_fld.B_part_buf + 1 + emf->nrow;
    } else emf->B_part = emf->B;
    if (e->mirrors) refresh_mirrors(e);
}

/* grid forms of emf_set_ext_fld / emf_init_fld for callers whose field
 * callbacks cannot return a float3 by value (e.g. Python through ctypes):
 * custom fields come as host grids in the reference layout, already
 * evaluated on every buffer cell */
EXPORT void emf_set_ext_fld_grid(t_emf *const emf, int E_type, const float E0[3], const float *E_grid,
                                 int B_type, const float B0[3], const float *B_grid)
{
    entry_t *e = need(reg_by_emf(emf), "emf_set_ext_fld_grid");
    if (E_type > EMF_FLD_TYPE_CUSTOM || B_type > EMF_FLD_TYPE_CUSTOM || E_type < 0 || B_type < 0)
        die("Invalid external field type, aborting.");
    zc_check(zc_set_ext_fld(e->gpu, E_type, E0, E_grid, B_type, B0, B_grid), "emf_set_ext_fld_grid");
    emf->ext_fld.E_type = (enum emf_fld_type)E_type;
    emf->ext_fld.B_type = (enum emf_fld_type)B_type;
    if (E0) emf->ext_fld.E_0 = (float3){E0[0], E0[1], E0[2]};
    if (B0) emf->ext_fld.B_0 = (float3){B0[0], B0[1], B0[2]};
    const size_t n = (size_t)emf->nrow * (emf->nx[1] + 3);
    if (E_type != EMF_FLD_TYPE_NONE) {
        if (!emf->ext_fld.E_part_buf) emf->ext_fld.E_part_buf = (float3 *)calloc(n, sizeof(float3));
        emf->E_part = emf->ext_fld.E_part_buf + 1 + emf->nrow;
    } else emf->E_part = emf->E;
    if (B_type != EMF_FLD_TYPE_NONE) {
        if (!emf->ext_fld.B_part_buf) emf->ext_fld.B_part_buf = (float3 *)calloc(n, sizeof(float3));
        emf->B_part = emf->ext_fld.B_part_buf + 1 + emf->nrow;
    } else emf->B_part = emf->B;
    if (e->mirrors) refresh_mirrors(e);
}

EXPORT void emf_init_fld_grid(t_emf *const emf, const float *E_grid, const float *B_grid)
{
    entry_t *e = need(reg_by_emf(emf), "emf_init_fld_grid");
    if (emf->iter != 0) die("emf_init_fld should only be called at initialization, aborting...");
    zc_check(zc_set_fields(e->gpu, E_grid, B_grid), "emf_init_fld_grid");
    if (e->mirrors) refresh_mirrors(e);
}

EXPORT void emf_init_fld(t_emf *const emf, t_emf_init_fld *init)
{
    entry_t *e = need(reg_by_emf(emf), "emf_init_fld");
    if (emf->iter != 0) die("emf_init_fld should only be called at initialization, aborting...");
    const int nrow = emf->nrow;
    zc_check(zc_get_fields(e->gpu, (float *)emf->E_buf, (float *)emf->B_buf), "emf_init_fld");
    for (int pass = 0; pass < 2; pass++) {
        const enum emf_fld_type t = pass ? init->B_type : init->E_type;
        if (t == EMF_FLD_TYPE_NONE) continue;
        float3 *F = pass ? emf->B : emf->E;
        for (int j = -1; j < emf->nx[1] + 2; j++)
            for (int i = -1; i < emf->nx[0] + 2; i++) {
                float3 v;
                if (t == EMF_FLD_TYPE_UNIFORM) v = pass ? init->B_0 : init->E_0;
                else if (pass) v = init->B_custom(i, emf->dx[0], j, emf->dx[1], init->B_custom_data);
                else v = init->E_custom(i, emf->dx[0], j, emf->dx[1], init->E_custom_data);
                F[j * nrow + i] = v;
            }
    }
    zc_check(zc_set_fields(e->gpu, (const float *)emf->E_buf, (const float *)emf->B_buf), "emf_init_fld");
    if (e->mirrors) refresh_mirrors(e);
}

/* ------------------------------------------------------------------------- */
/* host mirrors                                                              */
/* ------------------------------------------------------------------------- */
static void pull_species(entry_t *e, int k)
{
    t_species *sp = &e->sim->species[k];
    int np = 0;
    zc_check(zc_species_count(e->gpu, k, &np), "sync");
    spec_grow_buffer(sp, np);
    zc_check(zc_species_get_particles(e->gpu, k, (zc_part *)sp->part, sp->np_max, &np), "sync");
    sp->np = np;
}

static void sync_host(entry_t *e)
{
    t_simulation *sim = e->sim;
    zc_check(zc_get_fields(e->gpu, (float *)sim->emf.E_buf, (float *)sim->emf.B_buf), "sim_sync_host");
    if (sim->emf.ext_fld.E_part_buf || sim->emf.ext_fld.B_part_buf)
        zc_check(zc_get_particle_fields(e->gpu, (float *)sim->emf.ext_fld.E_part_buf,
                                        (float *)sim->emf.ext_fld.B_part_buf),
                 "sim_sync_host");
    zc_check(zc_get_current(e->gpu, (float *)sim->current.J_buf), "sim_sync_host");
    double emf_en[6];
    double *kin = (double *)calloc((size_t)(sim->n_species > 0 ? sim->n_species : 1), sizeof(double));
    zc_check(zc_energy(e->gpu, emf_en, kin), "sim_sync_host");
    for (int k = 0; k < sim->n_species; k++) {
        pull_species(e, k);
        sim->species[k].energy = kin[k];
    }
    free(kin);
}

EXPORT void sim_sync_host(t_simulation *sim)
{
    entry_t *e = need(reg_by_sim(sim), "sim_sync_host");
    sync_host(e);
    if (e->mirrors) shadow_save(e);
}

EXPORT zc_sim *sim_gpu_handle(t_simulation *sim)
{
    entry_t *e = reg_by_sim(sim);
    return e ? e->gpu : NULL;
}

EXPORT void sim_set_mirrors(t_simulation *sim, int every_step)
{
    entry_t *e = need(reg_by_sim(sim), "sim_set_mirrors");
    e->mirrors = every_step ? 1 : 0;
    if (e->mirrors) {
        refresh_mirrors(e);
        return;
    }
    if (e->shadow)  /* the remembered copies are not needed on demand */
        for (int k = 0; k < sim->n_species; k++) {
            free(e->shadow[k]);
            e->shadow[k] = NULL;
            e->shadow_np[k] = e->shadow_cap[k] = 0;
        }
    free(e->shadow_E);
    free(e->shadow_B);
    e->shadow_E = e->shadow_B = NULL;
}

EXPORT void sim_sync_device(t_simulation *sim)
{
    entry_t *e = need(reg_by_sim(sim), "sim_sync_device");
    zc_check(zc_set_fields(e->gpu, (const float *)sim->emf.E_buf, (const float *)sim->emf.B_buf),
             "sim_sync_device");
    for (int k = 0; k < sim->n_species; k++)
        zc_check(zc_species_set_particles(e->gpu, k, (const zc_part *)sim->species[k].part, sim->species[k].np),
                 "sim_sync_device");
    if (e->mirrors) shadow_save(e);
}

static void *xrealloc(void *p, size_t n)
{
    void *q = realloc(p, n ? n : 1);
    if (!q) die("(*error*) out of memory (host mirrors)");
    return q;
}

/* remembers every mirror as it is now (after a synchronisation) */
static void shadow_save(entry_t *e)
{
    t_simulation *sim = e->sim;
    const int ns = sim->n_species;
    if (!e->shadow) {
        e->shadow = (t_part **)calloc((size_t)(ns > 0 ? ns : 1), sizeof(t_part *));
        e->shadow_np = (int *)calloc((size_t)(ns > 0 ? ns : 1), sizeof(int));
        e->shadow_cap = (int *)calloc((size_t)(ns > 0 ? ns : 1), sizeof(int));
        if (!e->shadow || !e->shadow_np || !e->shadow_cap) die("(*error*) out of memory (host mirrors)");
    }
    for (int k = 0; k < ns; k++) {
        const t_species *sp = &sim->species[k];
        if (sp->np > e->shadow_cap[k]) {
            e->shadow[k] = (t_part *)xrealloc(e->shadow[k], (size_t)sp->np * sizeof(t_part));
            e->shadow_cap[k] = sp->np;
        }
        if (sp->np > 0) mirror_copy(e->shadow[k], sp->part, (size_t)sp->np * sizeof(t_part));
        e->shadow_np[k] = sp->np;
    }
    const size_t n = (size_t)sim->emf.nrow * (sim->emf.nx[1] + 3) * sizeof(float3);
    if (!e->shadow_E) e->shadow_E = (float3 *)xrealloc(NULL, n);
    if (!e->shadow_B) e->shadow_B = (float3 *)xrealloc(NULL, n);
    mirror_copy(e->shadow_E, sim->emf.E_buf, n);
    mirror_copy(e->shadow_B, sim->emf.B_buf, n);
}

/* uploads what the caller changed in the mirrors since they were last
 * synchronised: a species whose count or records differ, and E, B */
static void push_host_edits(entry_t *e)
{
    t_simulation *sim = e->sim;
    for (int k = 0; k < sim->n_species; k++) {
        const t_species *sp = &sim->species[k];
        if (sp->np != e->shadow_np[k] ||
            (sp->np > 0 && mirror_differs(sp->part, e->shadow[k], (size_t)sp->np * sizeof(t_part))))
            zc_check(zc_species_set_particles(e->gpu, k, (const zc_part *)sp->part, sp->np), "sim_iter");
    }
    const size_t n = (size_t)sim->emf.nrow * (sim->emf.nx[1] + 3) * sizeof(float3);
    if (mirror_differs(sim->emf.E_buf, e->shadow_E, n) || mirror_differs(sim->emf.B_buf, e->shadow_B, n))
        zc_check(zc_set_fields(e->gpu, (const float *)sim->emf.E_buf, (const float *)sim->emf.B_buf), "sim_iter");
}

/* every mirror refreshed from the device */
static void refresh_mirrors(entry_t *e)
{
    sync_host(e);
    shadow_save(e);
}

/* ------------------------------------------------------------------------- */
/* diagnostics                                                               */
/* ------------------------------------------------------------------------- */
EXPORT void emf_get_energy(const t_emf *emf, double energy[])
{
    entry_t *e = reg_by_emf(emf);
    if (!e) {  /* stand-alone field object: host computation (emf.c:729-750) */
        for (int i = 0; i < 6; i++) energy[i] = 0;
        for (int j = 0; j < emf->nx[1]; j++)
            for (int i = 0; i < emf->nx[0]; i++) {
                const float3 E = emf->E[i + j * emf->nrow], B = emf->B[i + j * emf->nrow];
                energy[0] += E.x * E.x;
                energy[1] += E.y * E.y;
                energy[2] += E.z * E.z;
                energy[3] += B.x * B.x;
                energy[4] += B.y * B.y;
                energy[5] += B.z * B.z;
            }
        for (int i = 0; i < 6; i++) energy[i] *= 0.5 * emf->dx[0] * emf->dx[1];
        return;
    }
    zc_check(zc_energy(e->gpu, energy, NULL), "emf_get_energy");
}

EXPORT void sim_report_energy(t_simulation *sim)
{
    entry_t *e = need(reg_by_sim(sim), "sim_report_energy");
    double en[6];
    double *kin = (double *)calloc((size_t)(sim->n_species > 0 ? sim->n_species : 1), sizeof(double));
    zc_check(zc_energy(e->gpu, en, kin), "sim_report_energy");
    /* the reference starts the field total at energy[0] and then adds all six
     * components (simulation.c:191-194); kept for identical output */
    double tot_emf = en[0];
    for (int i = 0; i < 6; i++) tot_emf += en[i];
    double tot_part = 0;
    for (int k = 0; k < sim->n_species; k++) {
        sim->species[k].energy = kin[k];
        tot_part += kin[k];
    }
    free(kin);
    printf("Energy (fields | particles | total) = %e %e %e\n", tot_emf, tot_part, tot_emf + tot_part);
}

EXPORT void spec_deposit_charge(const t_species *spec, float *charge)
{
    int k = 0;
    entry_t *e = reg_by_species(spec, &k);
    if (!e) {  /* species outside a simulation: host deposit (particles.c:1289-1324) */
        const int nrow = spec->nx[0] + 1;
        for (int i = 0; i < spec->np; i++) {
            const int c = spec->part[i].ix + nrow * spec->part[i].iy;
            const float w1 = spec->part[i].x, w2 = spec->part[i].y;
            charge[c] += (1.0f - w1) * (1.0f - w2) * spec->q;
            charge[c + 1] += w1 * (1.0f - w2) * spec->q;
            charge[c + nrow] += (1.0f - w1) * w2 * spec->q;
            charge[c + 1 + nrow] += w1 * w2 * spec->q;
        }
        if (!spec->moving_window)
            for (int j = 0; j < spec->nx[1] + 1; j++) charge[j * nrow] += charge[spec->nx[0] + j * nrow];
        for (int i = 0; i < spec->nx[0] + 1; i++) charge[i] += charge[i + spec->nx[1] * nrow];
        return;
    }
    zc_check(zc_species_charge(e->gpu, k, charge), "spec_deposit_charge");
}

/* phase-space density from the host mirror (particles.c:1512-1632) */
EXPORT void spec_deposit_pha(const t_species *spec, const int rep_type, const int pha_nx[],
                             const float pha_range[][2], float *buf)
{
    int k = 0;
    entry_t *e = reg_by_species(spec, &k);
    if (e) {  /* a species of a GPU simulation: deposited on the device */
        const float rg[4] = {pha_range[0][0], pha_range[0][1], pha_range[1][0], pha_range[1][1]};
        zc_check(zc_species_phasespace(e->gpu, k, rep_type & 0x000F, (rep_type & 0x00F0) >> 4, pha_nx, rg, buf),
                 "spec_deposit_pha");
        return;
    }
    /* a stand-alone species (no device state): on the host */
    const int nrow = pha_nx[0];
    const int q1 = rep_type & 0x000F, q2 = (rep_type & 0x00F0) >> 4;
    const float x1min = pha_range[0][0], x2min = pha_range[1][0];
    const float rdx1 = pha_nx[0] / (pha_range[0][1] - pha_range[0][0]);
    const float rdx2 = pha_nx[1] / (pha_range[1][1] - pha_range[1][0]);
    for (int n = 0; n < spec->np; n++) {
        const t_part *p = &spec->part[n];
        float a[2];
        for (int ax = 0; ax < 2; ax++) {
            const int qq = ax ? q2 : q1;
            a[ax] = (qq == X1) ? (p->x + p->ix) * spec->dx[0]
                  : (qq == X2) ? (p->y + p->iy) * spec->dx[1]
                  : (qq == U1) ? p->ux : (qq == U2) ? p->uy : p->uz;
        }
        const float nx1 = (a[0] - x1min) * rdx1, nx2 = (a[1] - x2min) * rdx2;
        const int i1 = (int)(nx1 + 0.5f), i2 = (int)(nx2 + 0.5f);
        const float w1 = nx1 - i1 + 0.5f, w2 = nx2 - i2 + 0.5f;
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

/* ------------------------------------------------------------------------- */
/* ZDF reports (emf.c:368-482, current.c:194-281, particles.c:1342-1750)     */
/* ------------------------------------------------------------------------- */
/* A report gathers its data -- fields and current straight from the device
 * buffers with an asynchronous copy of the one component asked for, charge,
 * phase space and particles through their host deposits -- and queues the
 * file for the background writer (zdf_io.c), so the simulation goes on
 * while the file is formatted and written.  zdf_flush() waits for the files. */
int zdf_async_submit(int (*run)(void *), void *arg);

/* page-locked buffers for the asynchronous copies, reused */
typedef struct pin_buf {
    void *p;
    size_t bytes;
    struct pin_buf *next;
} pin_buf;
static pthread_mutex_t pin_mu = PTHREAD_MUTEX_INITIALIZER;
static pin_buf *pin_free = NULL;
static int pin_nfree = 0;

static void *pin_get(size_t bytes, size_t *got)
{
    pthread_mutex_lock(&pin_mu);
    for (pin_buf **pp = &pin_free; *pp; pp = &(*pp)->next) {
        if ((*pp)->bytes >= bytes) {
            pin_buf *b = *pp;
            *pp = b->next;
            pin_nfree--;
            pthread_mutex_unlock(&pin_mu);
            void *p = b->p;
            *got = b->bytes;
            free(b);
            return p;
        }
    }
    pthread_mutex_unlock(&pin_mu);
    void *p = NULL;
    if (zc_host_alloc(bytes, &p) != ZC_OK) return NULL;
    *got = bytes;
    return p;
}

static void pin_put(void *p, size_t bytes)
{
    pin_buf *b = (pin_buf *)malloc(sizeof(pin_buf));
    pthread_mutex_lock(&pin_mu);
    if (!b || pin_nfree >= 8) {  /* keep a few for reuse */
        pthread_mutex_unlock(&pin_mu);
        free(b);
        zc_host_free(p);
        return;
    }
    b->p = p;
    b->bytes = bytes;
    b->next = pin_free;
    pin_free = b;
    pin_nfree++;
    pthread_mutex_unlock(&pin_mu);
}

static const char *const kUnitsX = "c/\\omega_p";
static const char *const kTimeUnits = "1/\\omega_p";

typedef struct grid_job {
    t_zdf_grid_info info;
    t_zdf_grid_axis axis[2];
    t_zdf_iteration iter;
    char name[128], label[128], units[64], path[1024];
    char ax_name[2][16], ax_label[2][16], ax_units[2][32];
    float *data;
    size_t bytes;  /* > 0: page-locked buffer of that size */
    zc_fence *fence;
} grid_job;

static int run_grid_job(void *arg)
{
    grid_job *j = (grid_job *)arg;
    int ok = 1;
    if (j->fence) {
        ok = zc_fence_wait(j->fence) == ZC_OK;
        zc_fence_destroy(j->fence);
    }
    if (ok) ok = zdf_save_grid(j->data, zdf_float32, &j->info, &j->iter, j->path);
    if (j->bytes) pin_put(j->data, j->bytes);
    else free(j->data);
    free(j);
    return ok;
}

/* a 2-D grid job with the reference's metadata layout */
static grid_job *grid_job_new(int nx, int ny, const char *units, double x0, double x1, double y0, double y1,
                              const char *axn0, const char *axl0, const char *axu0, const char *axn1,
                              const char *axl1, const char *axu1, int n, double t)
{
    grid_job *j = (grid_job *)calloc(1, sizeof(grid_job));
    if (!j) return NULL;
    snprintf(j->units, sizeof(j->units), "%s", units);
    snprintf(j->ax_name[0], 16, "%s", axn0);
    snprintf(j->ax_label[0], 16, "%s", axl0);
    snprintf(j->ax_units[0], 32, "%s", axu0);
    snprintf(j->ax_name[1], 16, "%s", axn1);
    snprintf(j->ax_label[1], 16, "%s", axl1);
    snprintf(j->ax_units[1], 32, "%s", axu1);
    for (int a = 0; a < 2; a++) {
        j->axis[a].name = j->ax_name[a];
        j->axis[a].type = zdf_linear;
        j->axis[a].label = j->ax_label[a];
        j->axis[a].units = j->ax_units[a];
    }
    j->axis[0].min = x0;
    j->axis[0].max = x1;
    j->axis[1].min = y0;
    j->axis[1].max = y1;
    j->info.name = j->name;
    j->info.ndims = 2;
    j->info.count[0] = (uint64_t)nx;
    j->info.count[1] = (uint64_t)ny;
    j->info.label = j->label;
    j->info.units = j->units;
    j->info.axis = j->axis;
    j->iter.name = "ITERATION";
    j->iter.n = n;
    j->iter.t = t;
    j->iter.time_units = (char *)kTimeUnits;
    return j;
}

/* the interior of component c of a host grid (float3, row stride nrow) */
static float *pack_component(const float3 *f, int nrow, int nx, int ny, int c)
{
    float *buf = (float *)malloc((size_t)nx * ny * sizeof(float));
    if (!buf) return NULL;
    for (int jy = 0; jy < ny; jy++)
        for (int ix = 0; ix < nx; ix++) {
            const float3 v = f[ix + jy * nrow];
            buf[ix + jy * nx] = (c == 0) ? v.x : (c == 1) ? v.y : v.z;
        }
    return buf;
}

/* fills job data: the device component when the grid belongs to a GPU
 * simulation, else the host one */
static int job_data(grid_job *j, entry_t *e, int grid, int comp, const float3 *host, int nrow, int nx, int ny)
{
    if (e) {
        size_t got = 0;
        j->data = (float *)pin_get((size_t)nx * ny * sizeof(float), &got);
        if (!j->data) return 0;
        j->bytes = got;
        if (zc_copy_grid_async(e->gpu, grid, comp, j->data, &j->fence) != ZC_OK) {
            pin_put(j->data, got);
            j->data = NULL;
            return 0;
        }
        return 1;
    }
    j->data = pack_component(host, nrow, nx, ny, comp);
    return j->data != NULL;
}

static void report_failed(grid_job *j, const char *what)
{
    fprintf(stderr, "(*error*) %s: %s\n", what, zc_last_error());
    free(j);
}

EXPORT void emf_report(const t_emf *emf, const char field, const int fc)
{
    static const char comp[] = {'x', 'y', 'z'};
    if (fc < 0 || fc > 2) {
        fprintf(stderr, "(*error*) Invalid field component (fc) selected, returning\n");
        return;
    }
    grid_job *j = grid_job_new(emf->nx[0], emf->nx[1], "m_e c \\omega_p e^{-1}", 0.0, emf->box[0], 0.0,
                               emf->box[1], "x", "x", kUnitsX, "y", "y", kUnitsX, emf->iter,
                               emf->iter * emf->dt);
    if (!j) return;
    int grid;
    const float3 *host;
    switch (field) {
    case EFLD:
        grid = ZC_GRID_E, host = emf->E;
        snprintf(j->name, 16, "E%1d", fc);
        snprintf(j->label, 16, "E_%c", comp[fc]);
        break;
    case BFLD:
        grid = ZC_GRID_B, host = emf->B;
        snprintf(j->name, 16, "B%1d", fc);
        snprintf(j->label, 16, "B_%c", comp[fc]);
        break;
    case EPART:
        grid = ZC_GRID_EPART, host = emf->E_part;
        snprintf(j->name, 16, "E%1d-part", fc);
        snprintf(j->label, 16, "E_{%cp}", comp[fc]);
        break;
    case BPART:
        grid = ZC_GRID_BPART, host = emf->B_part;
        snprintf(j->name, 16, "B%1d-part", fc);
        snprintf(j->label, 16, "B_{%cp}", comp[fc]);
        break;
    default:
        fprintf(stderr, "Invalid field type selected, returning\n");
        free(j);
        return;
    }
    snprintf(j->path, sizeof(j->path), "EMF");
    if (!job_data(j, reg_by_emf(emf), grid, fc, host, emf->nrow, emf->nx[0], emf->nx[1])) {
        report_failed(j, "emf_report");
        return;
    }
    zdf_async_submit(run_grid_job, j);
}

EXPORT void current_report(const t_current *current, const int jc)
{
    static const char comp[] = {'x', 'y', 'z'};
    if (jc < 0 || jc > 2) {
        fprintf(stderr, "(*error*) Invalid current component (jc) selected, returning\n");
        return;
    }
    grid_job *j = grid_job_new(current->nx[0], current->nx[1], "e \\omega_p^2 / c", 0.0, current->box[0], 0.0,
                               current->box[1], "x", "x", kUnitsX, "y", "y", kUnitsX, current->iter,
                               current->iter * current->dt);
    if (!j) return;
    snprintf(j->name, 3, "J%1u", (unsigned)jc);
    snprintf(j->label, 4, "J_%c", comp[jc]);
    snprintf(j->path, sizeof(j->path), "CURRENT");
    if (!job_data(j, reg_by_current(current), ZC_GRID_J, jc, current->J, current->nrow, current->nx[0],
                  current->nx[1])) {
        report_failed(j, "current_report");
        return;
    }
    zdf_async_submit(run_grid_job, j);
}

static void spec_rep_charge(const t_species *spec)
{
    const int nx = spec->nx[0], ny = spec->nx[1];
    float *charge = (float *)calloc((size_t)(nx + 1) * (ny + 1), sizeof(float));
    float *buf = (float *)malloc((size_t)nx * ny * sizeof(float));
    grid_job *j = grid_job_new(nx, ny, "n_e", spec->n_move * spec->dx[0], spec->box[0] + spec->n_move * spec->dx[0],
                               0.0, spec->box[1], "x", "x", kUnitsX, "y", "y", kUnitsX, spec->iter,
                               spec->iter * spec->dt);
    if (!charge || !buf || !j) {
        free(charge), free(buf), free(j);
        return;
    }
    spec_deposit_charge(spec, charge);
    for (int jy = 0; jy < ny; jy++) memcpy(buf + (size_t)jy * nx, charge + (size_t)jy * (nx + 1), nx * sizeof(float));
    free(charge);
    snprintf(j->name, sizeof(j->name), "%s-charge", spec->name);
    snprintf(j->label, sizeof(j->label), "%s \\rho", spec->name);
    snprintf(j->path, sizeof(j->path), "CHARGE/%s", spec->name);
    j->data = buf;
    zdf_async_submit(run_grid_job, j);
}

static const char *pha_units(int quant)
{
    switch (quant) {
    case X1:
    case X2:
        return "c/\\omega_p";
    case U1:
    case U2:
    case U3:
        return "m_e c";
    }
    return "";
}

static void spec_rep_pha(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2])
{
    static const char *const ax_name[] = {"x1", "x2", "x3", "u1", "u2", "u3"};
    static const char *const ax_label[] = {"x", "y", "z", "u_x", "u_y", "u_z"};
    const int q1 = rep_type & 0x000F, q2 = (rep_type & 0x00F0) >> 4;
    if (q1 < 1 || q1 > 6 || q2 < 1 || q2 > 6 || !pha_nx || !pha_range) {
        fprintf(stderr, "(*error*) Invalid phasespace type selected, returning\n");
        return;
    }
    float *buf = (float *)calloc((size_t)pha_nx[0] * pha_nx[1], sizeof(float));
    grid_job *j = grid_job_new(pha_nx[0], pha_nx[1], "a.u.", pha_range[0][0], pha_range[0][1], pha_range[1][0],
                               pha_range[1][1], ax_name[q1 - 1], ax_label[q1 - 1], pha_units(q1), ax_name[q2 - 1],
                               ax_label[q2 - 1], pha_units(q2), spec->iter, spec->iter * spec->dt);
    if (!buf || !j) {
        free(buf), free(j);
        return;
    }
    spec_deposit_pha(spec, rep_type, pha_nx, pha_range, buf);
    snprintf(j->name, 64, "%s-%s%s", spec->name, ax_name[q1 - 1], ax_name[q2 - 1]);
    snprintf(j->label, 64, "%s %s-%s", spec->name, ax_label[q1 - 1], ax_label[q2 - 1]);
    snprintf(j->path, sizeof(j->path), "PHASESPACE/%s", spec->name);
    j->data = buf;
    zdf_async_submit(run_grid_job, j);
}

typedef struct part_job {
    t_zdf_part_info info;
    t_zdf_iteration iter;
    char name[MAX_SPNAME_LEN + 1], path[1024];
    float *data;  /* x, y, ux, uy, uz, np each */
} part_job;

static int run_part_job(void *arg)
{
    static const char *const quants[] = {"x", "y", "ux", "uy", "uz"};
    part_job *j = (part_job *)arg;
    t_zdf_file f;
    int ok = zdf_open_part_file(&f, &j->info, &j->iter, j->path);
    for (int q = 0; ok && q < 5; q++)
        ok = zdf_add_quant_part_file(&f, quants[q], j->data + (size_t)q * j->info.np, j->info.np) || !j->info.np;
    if (f.fp) ok = zdf_close_file(&f) && ok;
    free(j->data);
    free(j);
    return ok;
}

static void spec_rep_particles(const t_species *spec)
{
    static const char *const quants[] = {"x", "y", "ux", "uy", "uz"};
    static const char *const qlabels[] = {"x", "y", "u_x", "u_y", "u_z"};
    static const char *const qunits[] = {"c/\\omega_p", "c/\\omega_p", "c", "c", "c"};
    int k = 0;
    entry_t *e = reg_by_species(spec, &k);
    if (e) pull_species(e, k);  /* refreshes the host mirror, as the particles go to the file */
    const size_t np = spec->np > 0 ? (size_t)spec->np : 0;
    part_job *j = (part_job *)calloc(1, sizeof(part_job));
    float *d = (float *)malloc(5 * (np ? np : 1) * sizeof(float));
    if (!j || !d) {
        free(j), free(d);
        return;
    }
    for (size_t i = 0; i < np; i++) {
        const t_part *p = &spec->part[i];
        d[i] = (spec->n_move + p->ix + p->x) * spec->dx[0];
        d[np + i] = (p->iy + p->y) * spec->dx[1];
        d[2 * np + i] = p->ux;
        d[3 * np + i] = p->uy;
        d[4 * np + i] = p->uz;
    }
    snprintf(j->name, sizeof(j->name), "%s", spec->name);
    snprintf(j->path, sizeof(j->path), "PARTICLES/%s", spec->name);
    j->info.name = j->name;
    j->info.label = j->name;
    j->info.np = np;
    j->info.nquants = 5;
    j->info.quants = (char **)quants;
    j->info.qlabels = (char **)qlabels;
    j->info.qunits = (char **)qunits;
    j->iter.name = "ITERATION";
    j->iter.n = spec->iter;
    j->iter.t = spec->iter * spec->dt;
    j->iter.time_units = (char *)kTimeUnits;
    j->data = d;
    zdf_async_submit(run_part_job, j);
}

EXPORT void spec_report(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2])
{
    switch (rep_type & 0xF000) {
    case CHARGE:
        spec_rep_charge(spec);
        break;
    case PHA:
        spec_rep_pha(spec, rep_type, pha_nx, pha_range);
        break;
    case PARTICLES:
        spec_rep_particles(spec);
        break;
    }
}

EXPORT void spec_move_window(t_species *spec)
{
    /* the GPU moves the window inside spec_advance / sim_iter; kept for API
     * completeness */
    (void)spec;
}
