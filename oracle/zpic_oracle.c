/*
 * zpic_oracle.c -- CPU restatement of the ZPIC em2d PIC step.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker for the CUDA path and is
 * never linked or called by the product.  See zpic_oracle.h for scope.
 *
 * Build with strict IEEE float32: -O2 -std=c99 -fno-fast-math
 * -ffp-contract=off (no FMA contraction), so that every operation rounds
 * exactly as the reference does when it is compiled the same way.
 */
#include "zpic_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI_2
#define M_PI_2 1.57079632679489661923132169163975144
#endif

/* ------------------------------------------------------------------------ */
/* Random numbers: em2d/random.c:16-101                                     */
/* ------------------------------------------------------------------------ */

/* Generator state is process-global in the reference (random.c:16-17) and
 * the cached second Box-Muller deviate (random.c:69-70) is NOT reset by
 * set_rand_seed; both facts are kept here. */
static uint32_t g_mw = 12345, g_mz = 67890;
static int g_have_spare = 0;
static double g_spare = 0.0;

void zo_set_rand_seed(uint32_t w, uint32_t z) { g_mw = w; g_mz = z; }   /* random.c:25-29 */

void zo_rand_fresh(void) { g_have_spare = 0; g_spare = 0.0; }

uint32_t zo_rand_uint32(void)                                              /* random.c:48-53 */
{
    g_mz = 36969u * (g_mz & 65535u) + (g_mz >> 16);
    g_mw = 18000u * (g_mw & 65535u) + (g_mw >> 16);
    return (g_mz << 16) + g_mw;
}

double zo_rand_norm(void)                                                  /* random.c:67-101 */
{
    if (g_have_spare) {
        g_have_spare = 0;
        return g_spare;
    }
    double a, b, r2;
    for (;;) {
        a = (zo_rand_uint32() + 0.5) / 2147483649.0 - 1.0;
        b = (zo_rand_uint32() + 0.5) / 2147483649.0 - 1.0;
        r2 = a * a + b * b;
        if (r2 != 0.0 && r2 < 1.0) break;
    }
    double f = sqrt(-2.0 * log(r2) / r2);
    g_spare = a * f;
    g_have_spare = 1;
    return b * f;
}

/* ------------------------------------------------------------------------ */
/* Data                                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
    char name[33];
    zo_part *p;
    int np, cap;
    float m_q, q;
    double energy;
    int ppc[2];
    zo_density dens;
    unsigned long cust_total_part;    /* particles.h:73-76 */
    double cust_total_q;
    float ufl[3], uth[3];
    int nx[2];
    float dx[2], box[2], dt;
    int iter, moving_window, n_move;
} zo_spec;

struct zo_sim {
    int nx[2], nrow, ncell_buf;
    float box[2], dx[2], dt;
    zo_f3 *Ebuf, *Bbuf, *Jbuf;        /* full buffers with guard cells */
    zo_f3 *E, *B, *J;                 /* cell (0,0) */
    zo_f3 *Epbuf, *Bpbuf;             /* particle fields when ext fields are on */
    zo_f3 *Ep, *Bp;
    int ext_E_type, ext_B_type;
    zo_f3 ext_E0, ext_B0;
    zo_field_fn ext_E_fn, ext_B_fn;
    void *ext_E_data, *ext_B_data;
    int smooth_xtype, smooth_ytype, smooth_xlevel, smooth_ylevel;
    int emf_iter, emf_n_move, cur_iter;
    int moving_window;
    int nspec;
    zo_spec *spec;
};

/* ------------------------------------------------------------------------ */
/* Species initialisation: em2d/particles.c:85-612                          */
/* ------------------------------------------------------------------------ */

static float unit_density(float x, void *d) { (void)x; (void)d; return 1.0f; }   /* particles.c:74-76 */

static void spec_reserve(zo_spec *sp, int want)                            /* particles.c:460-466 */
{
    if (want > sp->cap) {
        sp->cap = (want / 1024 + 1) * 1024;
        sp->p = (zo_part *)realloc(sp->p, (size_t)sp->cap * sizeof(zo_part));
    }
}

/* Thermal momenta, then per-cell mean removal, then the fluid drift.
 * particles.c:85-149 (the "#else" branch). */
static void spec_thermal_u(zo_spec *sp, int first, int last)
{
    for (int k = first; k <= last; k++) {
        sp->p[k].ux = sp->uth[0] * zo_rand_norm();
        sp->p[k].uy = sp->uth[1] * zo_rand_norm();
        sp->p[k].uz = sp->uth[2] * zo_rand_norm();
    }
    /* the reference indexes its per-cell table of nx[0]*nx[1] entries with
     * stride nx[1] (particles.c:104-105,116); kept as is.  With nx[1] >
     * nx[0] its indices run past the table (undefined behaviour there):
     * here the table is long enough for every index and all its entries
     * are normalised, i.e. the mean of each cell is removed.  With nx[1] <=
     * nx[0] this is the reference's arithmetic exactly. */
    const int stride = sp->nx[1];
    const int ncell = sp->nx[0] * sp->nx[1];
    const int nidx = (sp->nx[0] - 1) + stride * (sp->nx[1] - 1) + 1;
    const int ntab = nidx > ncell ? nidx : ncell;
    zo_f3 *mean = (zo_f3 *)calloc((size_t)ntab, sizeof(zo_f3));
    int *cnt = (int *)calloc((size_t)ntab, sizeof(int));
    for (int k = first; k <= last; k++) {
        int c = sp->p[k].ix + stride * sp->p[k].iy;
        mean[c].x += sp->p[k].ux;
        mean[c].y += sp->p[k].uy;
        mean[c].z += sp->p[k].uz;
        cnt[c] += 1;
    }
    for (int c = 0; c < ntab; c++) {
        float inv = (cnt[c] > 0) ? 1.0f / cnt[c] : 0;
        mean[c].x *= inv;
        mean[c].y *= inv;
        mean[c].z *= inv;
    }
    for (int k = first; k <= last; k++) {
        int c = sp->p[k].ix + stride * sp->p[k].iy;
        sp->p[k].ux += sp->ufl[0] - mean[c].x;
        sp->p[k].uy += sp->ufl[1] - mean[c].y;
        sp->p[k].uz += sp->ufl[2] - mean[c].z;
    }
    free(cnt);
    free(mean);
}

/* Upper bound of particles to inject in a cell range: particles.c:367-449 */
static int spec_count_inject(zo_spec *sp, const int r[2][2])
{
    int n = 0;
    switch (sp->dens.type) {
    case ZO_STEP: {
        int i0 = sp->dens.start / sp->dx[0] - sp->n_move;
        if (i0 > r[0][1]) n = 0;
        else {
            if (i0 < r[0][0]) i0 = r[0][0];
            n = (r[0][1] - i0 + 1) * sp->ppc[0];
        }
        n *= (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    } break;
    case ZO_SLAB: {
        int i0 = sp->dens.start / sp->dx[0] - sp->n_move;
        int i1 = sp->dens.end / sp->dx[1] - sp->n_move;   /* dx[1] as in particles.c:394 */
        if (i0 > r[0][1] || i1 < r[0][0]) n = 0;
        else {
            if (i0 < r[0][0]) i0 = r[0][0];
            if (i1 > r[0][1]) i1 = r[0][1];
            n = (i1 - i0 + 1) * sp->ppc[0];
        }
        n *= (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    } break;
    case ZO_CUSTOM: {
        double x = (r[0][0] + sp->n_move) * sp->dx[0];
        double qx = sp->dens.custom_x(x, sp->dens.custom_data_x);
        x = (r[0][1] + 1 + sp->n_move) * sp->dx[0];
        qx += sp->dens.custom_x(x, sp->dens.custom_data_x);
        qx *= 0.5;
        for (int i = r[0][0] + 1; i <= r[0][1]; i++) {
            x = (i + sp->n_move) * sp->dx[0];
            qx += sp->dens.custom_x(x, sp->dens.custom_data_x);
        }
        double y = r[1][0] * sp->dx[1];
        double qy = sp->dens.custom_y(y, sp->dens.custom_data_y);
        y = (r[1][1] + 1) * sp->dx[1];
        qy += sp->dens.custom_y(y, sp->dens.custom_data_y);
        qy *= 0.5;
        for (int j = r[1][0] + 1; j <= r[1][1]; j++) {
            y = j * sp->dx[1];
            qy += sp->dens.custom_y(y, sp->dens.custom_data_y);
        }
        n = ceil(qx * sp->ppc[0]) * ceil(qy * sp->ppc[1]);
    } break;
    case ZO_EMPTY:
        n = 0;
        break;
    default:
        n = (r[0][1] - r[0][0] + 1) * sp->ppc[0] * (r[1][1] - r[1][0] + 1) * sp->ppc[1];
    }
    return n;
}

/* Particle positions from the density profile: particles.c:159-354 */
static void spec_place(zo_spec *sp, const int r[2][2])
{
    const int npc = sp->ppc[0] * sp->ppc[1];
    const float hx = 1.0f / sp->ppc[0];
    const float hy = 1.0f / sp->ppc[1];
    float *cellpos = (float *)malloc(2 * (size_t)npc * sizeof(float));
    int m = 0;
    for (int b = 0; b < sp->ppc[1]; b++)
        for (int a = 0; a < sp->ppc[0]; a++) {
            cellpos[m] = hx * (a + 0.5);
            cellpos[m + 1] = hy * (b + 0.5);
            m += 2;
        }

    int n = sp->np;
    switch (sp->dens.type) {
    case ZO_STEP: {
        float edge = sp->dens.start / sp->dx[0] - sp->n_move;
        for (int j = r[1][0]; j <= r[1][1]; j++)
            for (int i = r[0][0]; i <= r[0][1]; i++)
                for (int k = 0; k < npc; k++)
                    if (i + cellpos[2 * k] > edge) {
                        sp->p[n].ix = i; sp->p[n].iy = j;
                        sp->p[n].x = cellpos[2 * k]; sp->p[n].y = cellpos[2 * k + 1];
                        n++;
                    }
    } break;
    case ZO_SLAB: {
        float lo = sp->dens.start / sp->dx[0] - sp->n_move;
        float hi = sp->dens.end / sp->dx[0] - sp->n_move;
        for (int j = r[1][0]; j <= r[1][1]; j++)
            for (int i = r[0][0]; i <= r[0][1]; i++)
                for (int k = 0; k < npc; k++)
                    if (i + cellpos[2 * k] > lo && i + cellpos[2 * k] < hi) {
                        sp->p[n].ix = i; sp->p[n].iy = j;
                        sp->p[n].x = cellpos[2 * k]; sp->p[n].y = cellpos[2 * k + 1];
                        n++;
                    }
    } break;
    case ZO_CUSTOM: {
        /* Inverse-CDF placement on the piecewise-linear density, continued
         * across moving-window injections through the running totals. */
        const double ddx = sp->dx[0], ddy = sp->dx[1];
        const double ux = 1.0 / sp->ppc[0], uy = 1.0 / sp->ppc[1];
        const double thr = 4 * ux * uy;
        const int mv = sp->n_move;
        const int i0 = r[0][0], j0 = r[1][0];
        unsigned long kx = sp->cust_total_part;
        double cum_hi_x = sp->cust_total_q, cum_lo_x;
        double nlo_x, nhi_x = sp->dens.custom_x((i0 + mv) * ddx, sp->dens.custom_data_x);
        const double nlo_y0 = sp->dens.custom_y(j0 * ddy, sp->dens.custom_data_y);
        for (int i = i0; i <= r[0][1]; i++) {
            nlo_x = nhi_x;
            nhi_x = sp->dens.custom_x((i + 1 + mv) * ddx, sp->dens.custom_data_x);
            cum_lo_x = cum_hi_x;
            cum_hi_x += 0.5 * (nlo_x + nhi_x);
            double tx;
            while ((tx = (kx + 0.5) * ux) < cum_hi_x) {
                double px = 2 * (tx - cum_lo_x) /
                            (sqrt(nlo_x * nlo_x + 2 * (nhi_x - nlo_x) * (tx - cum_lo_x)) + nlo_x);
                double dens_x = (0.5 - px) * nlo_x + (0.5 + px) * nhi_x;
                unsigned long ky = 0;
                double nlo_y, nhi_y = nlo_y0;
                double cum_lo_y, cum_hi_y = 0;
                for (int j = j0; j <= r[1][1]; j++) {
                    nlo_y = nhi_y;
                    nhi_y = sp->dens.custom_y((j + 1) * ddy, sp->dens.custom_data_y);
                    cum_lo_y = cum_hi_y;
                    cum_hi_y += 0.5 * (nlo_y + nhi_y);
                    double ty;
                    while ((ty = (ky + 0.5) * uy) < cum_hi_y) {
                        double py = 2 * (ty - cum_lo_y) /
                                    (sqrt(nlo_y * nlo_y + 2 * (nhi_y - nlo_y) * (ty - cum_lo_y)) + nlo_y);
                        double dens_y = (0.5 - py) * nlo_y + (0.5 + py) * nhi_y;
                        if (dens_x * dens_y > thr) {
                            sp->p[n].ix = i; sp->p[n].iy = j;
                            sp->p[n].x = px; sp->p[n].y = py;
                            n++;
                        }
                        ky++;
                    }
                }
                kx++;
            }
        }
        sp->cust_total_q = cum_hi_x;
        sp->cust_total_part = kx;
    } break;
    case ZO_EMPTY:
        break;
    default:
        for (int j = r[1][0]; j <= r[1][1]; j++)
            for (int i = r[0][0]; i <= r[0][1]; i++)
                for (int k = 0; k < npc; k++) {
                    sp->p[n].ix = i; sp->p[n].iy = j;
                    sp->p[n].x = cellpos[2 * k]; sp->p[n].y = cellpos[2 * k + 1];
                    n++;
                }
    }
    sp->np = n;
    free(cellpos);
}

static void spec_inject(zo_spec *sp, const int r[2][2])                    /* particles.c:476-492 */
{
    int first = sp->np;
    spec_reserve(sp, sp->np + spec_count_inject(sp, r));
    spec_place(sp, r);
    spec_thermal_u(sp, first, sp->np - 1);
}

int zo_sim_add_species(zo_sim *s, const char *name, float m_q, const int ppc[2],
                       const float *ufl, const float *uth, const zo_density *dens)
{
    s->spec = (zo_spec *)realloc(s->spec, (size_t)(s->nspec + 1) * sizeof(zo_spec));
    zo_spec *sp = &s->spec[s->nspec];
    memset(sp, 0, sizeof(*sp));
    strncpy(sp->name, name ? name : "", 32);
    int npc = 1;
    for (int d = 0; d < 2; d++) {                                           /* particles.c:546-555 */
        sp->nx[d] = s->nx[d];
        sp->ppc[d] = ppc[d];
        npc *= ppc[d];
        sp->box[d] = s->box[d];
        sp->dx[d] = s->box[d] / s->nx[d];
    }
    sp->m_q = m_q;
    sp->q = copysignf(1.0f, m_q) / npc;                                    /* particles.c:557 */
    sp->dt = s->dt;
    if (dens) sp->dens = *dens;
    else { memset(&sp->dens, 0, sizeof(sp->dens)); sp->dens.type = ZO_UNIFORM; sp->dens.n = 1.0f; }
    if (sp->dens.n == 0.) sp->dens.n = 1.0f;                               /* particles.c:499-517 */
    if (sp->dens.type == ZO_CUSTOM) {
        if (!sp->dens.custom_x) sp->dens.custom_x = unit_density;
        if (!sp->dens.custom_y) sp->dens.custom_y = unit_density;
        sp->cust_total_part = 0;
        sp->cust_total_q = 0;
    }
    sp->q *= fabsf(sp->dens.n);                                             /* particles.c:576 */
    for (int d = 0; d < 3; d++) {
        sp->ufl[d] = ufl ? ufl[d] : 0;
        sp->uth[d] = uth ? uth[d] : 0;
    }
    sp->iter = 0;
    sp->moving_window = 0;
    sp->n_move = 0;
    sp->np = 0;
    const int r[2][2] = {{0, s->nx[0] - 1}, {0, s->nx[1] - 1}};
    spec_inject(sp, r);
    return s->nspec++;
}

/* ------------------------------------------------------------------------ */
/* Particle push: em2d/particles.c:1029-1269                                */
/* ------------------------------------------------------------------------ */

/* Staggered bilinear field gather, particles.c:1029-1071 */
static void gather_fields(const zo_f3 *E, const zo_f3 *B, int nrow, const zo_part *p,
                          zo_f3 *e, zo_f3 *b)
{
    const int i = p->ix, j = p->iy;
    const float w1 = p->x, w2 = p->y;
    /* half-cell shifted stencil for the staggered components */
    const int ih = i + ((w1 < 0.5f) ? -1 : 0);
    const int jh = j + ((w2 < 0.5f) ? -1 : 0);
    const float w1h = w1 + ((w1 < 0.5f) ? 0.5f : -0.5f);
    const float w2h = w2 + ((w2 < 0.5f) ? 0.5f : -0.5f);

#define LERP2(F, c, a0, b0, wa, wb)                                                        \
    ((F[(a0) + (b0)*nrow].c * (1.0f - (wa)) + F[(a0) + 1 + (b0)*nrow].c * (wa)) * (1.0f - (wb)) + \
     (F[(a0) + ((b0) + 1) * nrow].c * (1.0f - (wa)) + F[(a0) + 1 + ((b0) + 1) * nrow].c * (wa)) * (wb))

    e->x = LERP2(E, x, ih, j, w1h, w2);
    e->y = LERP2(E, y, i, jh, w1, w2h);
    e->z = LERP2(E, z, i, j, w1, w2);
    b->x = LERP2(B, x, i, jh, w1, w2h);
    b->y = LERP2(B, y, ih, j, w1h, w2);
    b->z = LERP2(B, z, ih, jh, w1h, w2h);
#undef LERP2
}

/* ltrim, particles.c:1081-1084 */
static int cell_shift(float x) { return (x >= 1.0f) - (x < 0.0f); }

typedef struct { float x0, x1, y0, y1, dx, dy, qvz; int ix, iy; } vseg;

/* Charge-conserving zigzag deposit, particles.c:773-924.  The trajectory is
 * cut at the x crossing, then at the y crossing, into at most three
 * straight segments, each depositing inside one cell. */
static void deposit_zigzag(zo_f3 *J, int nrow, int ix, int iy, int di, int dj,
                           float x0, float y0, float dx, float dy,
                           float qnx, float qny, float qvz)
{
    vseg v[3];
    int n = 1;
    v[0].x0 = x0; v[0].y0 = y0;
    v[0].dx = dx; v[0].dy = dy;
    v[0].x1 = x0 + dx; v[0].y1 = y0 + dy;
    v[0].qvz = qvz / 2.0;
    v[0].ix = ix; v[0].iy = iy;

    if (di != 0) {                                     /* particles.c:805-839 */
        const int xb = (di == 1);
        const float f = (x0 + dx - xb) / dx;           /* part of the motion past the edge */
        const float yc = y0 + dy * (1.0f - f);
        v[1].x0 = 1 - xb;
        v[1].x1 = (x0 + dx) - di;
        v[1].dx = dx * f;
        v[1].ix = ix + di;
        v[1].y0 = yc;
        v[1].y1 = v[0].y1;
        v[1].dy = dy * f;
        v[1].iy = iy;
        v[1].qvz = v[0].qvz * f;
        v[0].x1 = xb;
        v[0].dx *= (1.0f - f);
        v[0].dy *= (1.0f - f);
        v[0].y1 = yc;
        v[0].qvz *= (1.0f - f);
        n++;
    }
    if (dj != 0) {                                     /* particles.c:842-879 */
        /* segment that actually crosses the y edge */
        const int c = 1 - (v[0].y1 < 0.0f || v[0].y1 >= 1.0f);
        const int yb = (dj == 1);
        const float f = (v[c].y1 - yb) / v[c].dy;
        const float xc = v[c].x0 + v[c].dx * (1.0f - f);
        v[n].y0 = 1 - yb;
        v[n].y1 = v[c].y1 - dj;
        v[n].dy = v[c].dy * f;
        v[n].iy = v[c].iy + dj;
        v[n].x0 = xc;
        v[n].x1 = v[c].x1;
        v[n].dx = v[c].dx * f;
        v[n].ix = v[c].ix;
        v[n].qvz = v[c].qvz * f;
        v[c].y1 = yb;
        v[c].dy *= (1.0f - f);
        v[c].dx *= (1.0f - f);
        v[c].x1 = xc;
        v[c].qvz *= (1.0f - f);
        if (c < n - 1) {            /* the x-split tail lies wholly past the y edge */
            v[1].y0 -= dj;
            v[1].y1 -= dj;
            v[1].iy += dj;
        }
        n++;
    }

    for (int k = 0; k < n; k++) {                      /* particles.c:886-922 */
        const float s0x0 = 1.0f - v[k].x0, s0x1 = v[k].x0;
        const float s1x0 = 1.0f - v[k].x1, s1x1 = v[k].x1;
        const float s0y0 = 1.0f - v[k].y0, s0y1 = v[k].y0;
        const float s1y0 = 1.0f - v[k].y1, s1y1 = v[k].y1;
        const float jx = qnx * v[k].dx;
        const float jy = qny * v[k].dy;
        const float ay0 = 0.5f * (s0y0 + s1y0), ay1 = 0.5f * (s0y1 + s1y1);
        const float ax0 = 0.5f * (s0x0 + s1x0), ax1 = 0.5f * (s0x1 + s1x1);
        const int c00 = v[k].ix + nrow * v[k].iy;
        J[c00].x += jx * ay0;
        J[c00 + nrow].x += jx * ay1;
        J[c00].y += jy * ax0;
        J[c00 + 1].y += jy * ax1;
        const float q = v[k].qvz;
        J[c00].z += q * (s0x0 * s0y0 + s1x0 * s1y0 + (s0x0 * s1y0 - s1x0 * s0y0) / 2.0f);
        J[c00 + 1].z += q * (s0x1 * s0y0 + s1x1 * s1y0 + (s0x1 * s1y0 - s1x1 * s0y0) / 2.0f);
        J[c00 + nrow].z += q * (s0x0 * s0y1 + s1x0 * s1y1 + (s0x0 * s1y1 - s1x0 * s0y1) / 2.0f);
        J[c00 + 1 + nrow].z += q * (s0x1 * s0y1 + s1x1 * s1y1 + (s0x1 * s1y1 - s1x1 * s0y1) / 2.0f);
    }
}

/* spec_move_window, particles.c:619-640 */
static void spec_window(zo_spec *sp)
{
    if ((sp->iter * sp->dt) > (sp->dx[0] * (sp->n_move + 1))) {
        for (int k = 0; k < sp->np; k++) sp->p[k].ix--;
        sp->n_move++;
        const int r[2][2] = {{sp->nx[0] - 1, sp->nx[0] - 1}, {0, sp->nx[1] - 1}};
        spec_inject(sp, r);
    }
}

void zo_spec_advance(zo_sim *s, int si)                                   /* particles.c:1104-1269 */
{
    zo_spec *sp = &s->spec[si];
    const float tem = 0.5 * sp->dt / sp->m_q;
    const float dt_dx = sp->dt / sp->dx[0];
    const float dt_dy = sp->dt / sp->dx[1];
    const float qnx = sp->q * sp->dx[0] / sp->dt;
    const float qny = sp->q * sp->dx[1] / sp->dt;
    const int nx0 = sp->nx[0], nx1 = sp->nx[1];
    double ekin = 0;

    for (int k = 0; k < sp->np; k++) {
        zo_part *p = &sp->p[k];
        zo_f3 e, b;
        float ux = p->ux, uy = p->uy, uz = p->uz;
        gather_fields(s->Ep, s->Bp, s->nrow, p, &e, &b);

        /* Boris: half electric kick, magnetic rotation, half kick
         * (particles.c:1145-1187) */
        e.x *= tem; e.y *= tem; e.z *= tem;
        float tx = ux + e.x, ty = uy + e.y, tz = uz + e.z;
        const float u2 = tx * tx + ty * ty + tz * tz;
        const float g = sqrtf(1.0f + u2);
        ekin += u2 / (g + 1);
        const float tg = tem / g;
        b.x *= tg; b.y *= tg; b.z *= tg;
        const float s2 = 2.0f / (1.0f + b.x * b.x + b.y * b.y + b.z * b.z);
        ux = tx + ty * b.z - tz * b.y;
        uy = ty + tz * b.x - tx * b.z;
        uz = tz + tx * b.y - ty * b.x;
        b.x *= s2; b.y *= s2; b.z *= s2;
        tx += uy * b.z - uz * b.y;
        ty += uz * b.x - ux * b.z;
        tz += ux * b.y - uy * b.x;
        ux = tx + e.x; uy = ty + e.y; uz = tz + e.z;
        p->ux = ux; p->uy = uy; p->uz = uz;

        /* move (particles.c:1194-1207) */
        const float rg = 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
        const float mx = dt_dx * rg * ux;
        const float my = dt_dy * rg * uy;
        float x1 = p->x + mx, y1 = p->y + my;
        const int di = cell_shift(x1), dj = cell_shift(y1);
        x1 -= di;
        y1 -= dj;
        const float qvz = sp->q * uz * rg;
        deposit_zigzag(s->J, s->nrow, p->ix, p->iy, di, dj, p->x, p->y, mx, my, qnx, qny, qvz);
        p->x = x1;
        p->y = y1;
        p->ix += di;
        p->iy += dj;
    }
    sp->energy = sp->q * sp->m_q * ekin * sp->dx[0] * sp->dx[1];            /* particles.c:1231 */
    sp->iter += 1;

    if (sp->moving_window) {                                                /* particles.c:1234-1251 */
        spec_window(sp);
        int k = 0;
        while (k < sp->np) {
            if (sp->p[k].ix < 0 || sp->p[k].ix >= nx0) {
                sp->p[k] = sp->p[--sp->np];
                continue;
            }
            sp->p[k].iy += ((sp->p[k].iy < 0) ? nx1 : 0) - ((sp->p[k].iy >= nx1) ? nx1 : 0);
            k++;
        }
    } else {                                                                /* particles.c:1253-1259 */
        for (int k = 0; k < sp->np; k++) {
            sp->p[k].ix += ((sp->p[k].ix < 0) ? nx0 : 0) - ((sp->p[k].ix >= nx0) ? nx0 : 0);
            sp->p[k].iy += ((sp->p[k].iy < 0) ? nx1 : 0) - ((sp->p[k].iy >= nx1) ? nx1 : 0);
        }
    }
    /* spec_sort (particles.c:942-1007, every n_sort steps) only reorders the
     * buffer; it is a cache optimisation and does not change the physics,
     * so the oracle keeps buffer order. */
}

/* ------------------------------------------------------------------------ */
/* Current: em2d/current.c:98-459                                           */
/* ------------------------------------------------------------------------ */

void zo_current_zero(zo_sim *s)                                            /* current.c:98-107 */
{
    memset(s->Jbuf, 0, (size_t)s->ncell_buf * sizeof(zo_f3));
}

/* Periodic guard fold: current.c:118-159 */
static void current_fold(zo_sim *s)
{
    const int nrow = s->nrow, nx = s->nx[0], ny = s->nx[1];
    zo_f3 *J = s->J;
    if (!s->moving_window) {
        for (int j = -1; j < ny + 2; j++) {
            for (int i = -1; i < 2; i++) {
                J[i + j * nrow].x += J[nx + i + j * nrow].x;
                J[i + j * nrow].y += J[nx + i + j * nrow].y;
                J[i + j * nrow].z += J[nx + i + j * nrow].z;
            }
            for (int i = -1; i < 2; i++) J[nx + i + j * nrow] = J[i + j * nrow];
        }
    }
    for (int i = -1; i < nx + 2; i++) {
        for (int j = -1; j < 2; j++) {
            J[i + j * nrow].x += J[i + (ny + j) * nrow].x;
            J[i + j * nrow].y += J[i + (ny + j) * nrow].y;
            J[i + j * nrow].z += J[i + (ny + j) * nrow].z;
        }
        for (int j = -1; j < 2; j++) J[i + (ny + j) * nrow] = J[i + j * nrow];
    }
}

/* compensator [a,b,a] for n binomial passes, current.c:297-304 */
static void smooth_comp(int n, float *sa, float *sb)
{
    float a = -1;
    float b = (4.0 + 2.0 * n) / n;
    float t = 2 * a + b;
    *sa = a / t;
    *sb = b / t;
}

/* 3-point filter along x, current.c:316-354 */
static void filter_x(zo_sim *s, float sa, float sb)
{
    const int nrow = s->nrow, nx = s->nx[0], ny = s->nx[1];
    zo_f3 *J = s->J;
    for (int j = 0; j < ny; j++) {
        zo_f3 *row = J + j * nrow;
        zo_f3 lo = row[-1], mid = row[0];
        for (int i = 0; i < nx; i++) {
            zo_f3 hi = row[i + 1], o;
            o.x = sa * lo.x + sb * mid.x + sa * hi.x;
            o.y = sa * lo.y + sb * mid.y + sa * hi.y;
            o.z = sa * lo.z + sb * mid.z + sa * hi.z;
            row[i] = o;
            lo = mid;
            mid = hi;
        }
        if (!s->moving_window) {
            row[-1] = row[nx - 1];
            for (int i = 0; i < 2; i++) row[nx + i] = row[i];
        }
    }
}

/* 3-point filter along y, current.c:366-413 */
static void filter_y(zo_sim *s, float sa, float sb)
{
    const int nrow = s->nrow, nx = s->nx[0], ny = s->nx[1];
    zo_f3 *J = s->J;
    zo_f3 *prev = (zo_f3 *)malloc((size_t)nx * sizeof(zo_f3));
    for (int i = 0; i < nx; i++) prev[i] = J[i - nrow];
    for (int j = 0; j < ny; j++) {
        for (int i = 0; i < nx; i++) {
            zo_f3 lo = prev[i], mid = J[j * nrow + i], hi = J[(j + 1) * nrow + i], o;
            prev[i] = mid;
            o.x = sa * lo.x + sb * mid.x + sa * hi.x;
            o.y = sa * lo.y + sb * mid.y + sa * hi.y;
            o.z = sa * lo.z + sb * mid.z + sa * hi.z;
            J[j * nrow + i] = o;
        }
    }
    free(prev);
    for (int i = -1; i < nx + 2; i++) {
        J[i - nrow] = J[i + (ny - 1) * nrow];
        for (int j = 0; j < 2; j++) J[i + (ny + j) * nrow] = J[i + j * nrow];
    }
}

/* current_smooth, current.c:427-459.  The y binomial pass count is xlevel,
 * exactly as in the reference (current.c:449). */
static void current_filter(zo_sim *s)
{
    float sa, sb;
    if (s->smooth_xtype != ZO_SMOOTH_NONE) {
        for (int k = 0; k < s->smooth_xlevel; k++) filter_x(s, 0.25, 0.5);
        if (s->smooth_xtype == ZO_SMOOTH_COMPENSATED) {
            smooth_comp(s->smooth_xlevel, &sa, &sb);
            filter_x(s, sa, sb);
        }
    }
    if (s->smooth_ytype != ZO_SMOOTH_NONE) {
        for (int k = 0; k < s->smooth_xlevel; k++) filter_y(s, 0.25, 0.5);
        if (s->smooth_ytype == ZO_SMOOTH_COMPENSATED) {
            smooth_comp(s->smooth_ylevel, &sa, &sb);
            filter_y(s, sa, sb);
        }
    }
}

void zo_current_update(zo_sim *s)                                          /* current.c:171-183 */
{
    current_fold(s);
    current_filter(s);
    s->cur_iter++;
}

/* ------------------------------------------------------------------------ */
/* Fields: em2d/emf.c                                                       */
/* ------------------------------------------------------------------------ */

/* B half step, emf.c:500-522 */
static void yee_half_b(zo_sim *s, float dt)
{
    const int nrow = s->nrow;
    const float cx = dt / s->dx[0], cy = dt / s->dx[1];
    zo_f3 *B = s->B;
    const zo_f3 *E = s->E;
    for (int j = -1; j <= s->nx[1]; j++)
        for (int i = -1; i <= s->nx[0]; i++) {
            const int c = i + j * nrow;
            B[c].x += (-cy * (E[c + nrow].z - E[c].z));
            B[c].y += (cx * (E[c + 1].z - E[c].z));
            B[c].z += (-cx * (E[c + 1].y - E[c].y) + cy * (E[c + nrow].x - E[c].x));
        }
}

/* E full step, emf.c:531-562 */
static void yee_full_e(zo_sim *s, float dt)
{
    const int nrow = s->nrow;
    const float cx = dt / s->dx[0], cy = dt / s->dx[1];
    zo_f3 *E = s->E;
    const zo_f3 *B = s->B, *J = s->J;
    for (int j = 0; j <= s->nx[1] + 1; j++)
        for (int i = 0; i <= s->nx[0] + 1; i++) {
            const int c = i + j * nrow;
            E[c].x += (+cy * (B[c].z - B[c - nrow].z)) - dt * J[c].x;
            E[c].y += (-cx * (B[c].z - B[c - 1].z)) - dt * J[c].y;
            E[c].z += (+cx * (B[c].y - B[c - 1].y) - cy * (B[c].x - B[c - nrow].x)) - dt * J[c].z;
        }
}

/* Periodic guard cells, emf.c:573-637 */
static void emf_guards(zo_sim *s)
{
    const int nrow = s->nrow, nx = s->nx[0], ny = s->nx[1];
    zo_f3 *E = s->E, *B = s->B;
    if (!s->moving_window) {
        for (int j = -1; j < ny + 2; j++) {
            const int r = j * nrow;
            E[-1 + r] = E[nx - 1 + r];
            B[-1 + r] = B[nx - 1 + r];
            for (int i = 0; i < 2; i++) {
                E[nx + i + r] = E[i + r];
                B[nx + i + r] = B[i + r];
            }
        }
    }
    for (int i = -1; i < nx + 2; i++) {
        E[i - nrow] = E[i + (ny - 1) * nrow];
        B[i - nrow] = B[i + (ny - 1) * nrow];
        for (int j = 0; j < 2; j++) {
            E[i + (ny + j) * nrow] = E[i + j * nrow];
            B[i + (ny + j) * nrow] = B[i + j * nrow];
        }
    }
}

/* Window shift of the fields, emf.c:648-675 */
static void emf_window(zo_sim *s)
{
    if ((s->emf_iter * s->dt) > s->dx[0] * (s->emf_n_move + 1)) {
        const int nrow = s->nrow, nx = s->nx[0], ny = s->nx[1];
        const zo_f3 z = {0, 0, 0};
        for (int j = -1; j < ny + 2; j++) {
            zo_f3 *E = s->E + j * nrow, *B = s->B + j * nrow;
            for (int i = -1; i < nx + 1; i++) {
                E[i] = E[i + 1];
                B[i] = B[i + 1];
            }
            for (int i = nx - 1; i < nx + 2; i++) {
                E[i] = z;
                B[i] = z;
            }
        }
        s->emf_n_move++;
    }
}

/* E_part / B_part with external fields, emf.c:838-914 */
static void emf_particle_fields(zo_sim *s)
{
    const int nrow = s->nrow;
    for (int pass = 0; pass < 2; pass++) {
        const int type = pass ? s->ext_B_type : s->ext_E_type;
        if (type == ZO_FLD_NONE) continue;
        const zo_f3 *F = pass ? s->B : s->E;
        zo_f3 *P = pass ? s->Bp : s->Ep;
        for (int j = -1; j < s->nx[1] + 2; j++)
            for (int i = -1; i < s->nx[0] + 2; i++) {
                zo_f3 add;
                if (type == ZO_FLD_UNIFORM) add = pass ? s->ext_B0 : s->ext_E0;
                else {
                    float o[3];
                    if (pass) s->ext_B_fn(i, s->dx[0], j, s->dx[1], s->ext_B_data, o);
                    else s->ext_E_fn(i, s->dx[0], j, s->dx[1], s->ext_E_data, o);
                    add.x = o[0]; add.y = o[1]; add.z = o[2];
                }
                zo_f3 v = F[i + j * nrow];
                v.x += add.x; v.y += add.y; v.z += add.z;
                P[i + j * nrow] = v;
            }
    }
}

void zo_emf_advance(zo_sim *s)                                             /* emf.c:688-716 */
{
    const float dt = s->dt;
    yee_half_b(s, dt / 2.0f);
    yee_full_e(s, dt);
    yee_half_b(s, dt / 2.0f);
    emf_guards(s);
    emf_particle_fields(s);
    s->emf_iter += 1;
    if (s->moving_window) emf_window(s);
}

void zo_emf_energy(const zo_sim *s, double en[6])                          /* emf.c:729-750 */
{
    const int nrow = s->nrow;
    for (int k = 0; k < 6; k++) en[k] = 0;
    for (int j = 0; j < s->nx[1]; j++)
        for (int i = 0; i < s->nx[0]; i++) {
            const zo_f3 e = s->E[i + j * nrow], b = s->B[i + j * nrow];
            en[0] += e.x * e.x;
            en[1] += e.y * e.y;
            en[2] += e.z * e.z;
            en[3] += b.x * b.x;
            en[4] += b.y * b.y;
            en[5] += b.z * b.z;
        }
    for (int k = 0; k < 6; k++) en[k] *= 0.5 * s->dx[0] * s->dx[1];
}

/* ---- laser pulses, emf.c:158-350 ---- */

static float laser_gauss(const zo_laser *L, float zpos, float r)            /* emf.c:158-170 */
{
    float z = zpos - L->focus;
    float zr = L->omega0 * (L->W0 * L->W0) / 2;
    float r2 = r * r;
    float curv = r2 * z / (zr * zr + z * z);
    float w2r = (zr * zr) / (zr * zr + z * z);
    float gouy = atan2(z, zr);
    return sqrt(sqrt(w2r)) * exp(-r2 * w2r / (L->W0 * L->W0)) * cos(L->omega0 * (z + curv) - gouy);
}

static float laser_envelope(const zo_laser *L, float z)                    /* emf.c:179-202 */
{
    if (z > L->start) return 0.0;
    if (z > L->start - L->rise) {
        float u = z - L->start;
        float e = sin(M_PI_2 * u / L->rise);
        return e * e;
    }
    if (z > L->start - (L->rise + L->flat)) return 1.0;
    if (z > L->start - (L->rise + L->flat + L->fall)) {
        float u = z - (L->start - L->rise - L->flat - L->fall);
        float e = sin(M_PI_2 * u / L->fall);
        return e * e;
    }
    return 0.0;
}

static void laser_div_clean(zo_sim *s)                                      /* emf.c:213-231 */
{
    const int nrow = s->nrow;
    const double rxy = s->dx[0] / s->dx[1];
    for (int j = 0; j < s->nx[1]; j++) {
        double ex = 0.0, bx = 0.0;
        for (int i = s->nx[0] - 1; i >= 0; i--) {
            ex += rxy * (s->E[i + 1 + j * nrow].y - s->E[i + 1 + (j - 1) * nrow].y);
            s->E[i + j * nrow].x = ex;
            bx += rxy * (s->B[i + (j + 1) * nrow].y - s->B[i + j * nrow].y);
            s->B[i + j * nrow].x = bx;
        }
    }
}

int zo_sim_add_laser(zo_sim *s, const zo_laser *Lin)                       /* emf.c:242-350 */
{
    zo_laser L = *Lin;
    if (L.fwhm != 0) {
        if (L.fwhm <= 0) return -1;
        L.rise = L.fwhm;
        L.fall = L.fwhm;
        L.flat = 0.;
    }
    if (L.rise <= 0 || L.flat < 0 || L.fall <= 0) return -1;

    const int nrow = s->nrow;
    const float dx = s->dx[0], dy = s->dx[1];
    const float amp = L.omega0 * L.a0;
    const float cp = cos(L.polarization), sp = sin(L.polarization);
    zo_f3 *E = s->E, *B = s->B;
    if (L.type == 0) {
        const float k = L.omega0;
        for (int i = 0; i < s->nx[0]; i++) {
            const float z = i * dx, z2 = z + dx / 2;
            const float a = amp * laser_envelope(&L, z), a2 = amp * laser_envelope(&L, z2);
            for (int j = 0; j < s->nx[1]; j++) {
                E[i + j * nrow].y += +a * cos(k * z) * cp;
                E[i + j * nrow].z += +a * cos(k * z) * sp;
                B[i + j * nrow].y += -a2 * cos(k * z2) * sp;
                B[i + j * nrow].z += +a2 * cos(k * z2) * cp;
            }
        }
    } else if (L.type == 1) {
        for (int i = 0; i < s->nx[0]; i++) {
            const float z = i * dx, z2 = z + dx / 2;
            const float a = amp * laser_envelope(&L, z), a2 = amp * laser_envelope(&L, z2);
            for (int j = 0; j < s->nx[1]; j++) {
                const float r = j * dy - L.axis, r2 = r + dy / 2;
                E[i + j * nrow].y += +a * laser_gauss(&L, z, r2) * cp;
                E[i + j * nrow].z += +a * laser_gauss(&L, z, r) * sp;
                B[i + j * nrow].y += -a2 * laser_gauss(&L, z2, r) * sp;
                B[i + j * nrow].z += +a2 * laser_gauss(&L, z2, r2) * cp;
            }
        }
        laser_div_clean(s);
    }
    emf_guards(s);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Simulation object: em2d/simulation.c                                     */
/* ------------------------------------------------------------------------ */

zo_sim *zo_sim_new(const int nx[2], const float box[2], float dt, char *err, int errlen)
{
    zo_sim *s = (zo_sim *)calloc(1, sizeof(zo_sim));
    for (int d = 0; d < 2; d++) {
        s->nx[d] = nx[d];
        s->box[d] = box[d];
        s->dx[d] = box[d] / nx[d];
    }
    s->dt = dt;
    s->nrow = nx[0] + 3;
    s->ncell_buf = (nx[0] + 3) * (nx[1] + 3);
    s->Ebuf = (zo_f3 *)calloc((size_t)s->ncell_buf, sizeof(zo_f3));
    s->Bbuf = (zo_f3 *)calloc((size_t)s->ncell_buf, sizeof(zo_f3));
    s->Jbuf = (zo_f3 *)calloc((size_t)s->ncell_buf, sizeof(zo_f3));
    s->E = s->Ebuf + 1 + s->nrow;
    s->B = s->Bbuf + 1 + s->nrow;
    s->J = s->Jbuf + 1 + s->nrow;
    s->Ep = s->E;
    s->Bp = s->B;
    /* Courant condition, simulation.c:105-110 */
    float cour = sqrtf(1.0f / (1.0f / (s->dx[0] * s->dx[0]) + 1.0f / (s->dx[1] * s->dx[1])));
    if (dt >= cour) {
        if (err) snprintf(err, (size_t)errlen, "Invalid timestep, courant condition violation, dtmax = %f", cour);
        zo_sim_delete(s);
        return NULL;
    }
    return s;
}

void zo_sim_delete(zo_sim *s)
{
    if (!s) return;
    for (int k = 0; k < s->nspec; k++) free(s->spec[k].p);
    free(s->spec);
    free(s->Ebuf); free(s->Bbuf); free(s->Jbuf);
    free(s->Epbuf); free(s->Bpbuf);
    free(s);
}

int zo_sim_set_smooth(zo_sim *s, int xtype, int xlevel, int ytype, int ylevel)   /* simulation.c:134-147 */
{
    if (xtype != ZO_SMOOTH_NONE && xlevel <= 0) return -1;
    if (ytype != ZO_SMOOTH_NONE && ylevel <= 0) return -1;
    s->smooth_xtype = xtype; s->smooth_xlevel = xlevel;
    s->smooth_ytype = ytype; s->smooth_ylevel = ylevel;
    return 0;
}

void zo_sim_set_moving_window(zo_sim *s)                                   /* simulation.c:154-163 */
{
    s->moving_window = 1;
    for (int k = 0; k < s->nspec; k++) s->spec[k].moving_window = 1;
}

static int set_part_grid(zo_sim *s, int pass, int type, const float v0[3], zo_field_fn fn, void *data)
{
    if (type == ZO_FLD_NONE) {
        if (pass) { s->Bp = s->B; } else { s->Ep = s->E; }
        if (pass) s->ext_B_type = ZO_FLD_NONE; else s->ext_E_type = ZO_FLD_NONE;
        return 0;
    }
    if (type != ZO_FLD_UNIFORM && type != ZO_FLD_CUSTOM) return -1;
    zo_f3 **buf = pass ? &s->Bpbuf : &s->Epbuf;
    if (!*buf) *buf = (zo_f3 *)calloc((size_t)s->ncell_buf, sizeof(zo_f3));
    if (pass) {
        s->ext_B_type = type; s->Bp = s->Bpbuf + 1 + s->nrow;
        if (v0) { s->ext_B0.x = v0[0]; s->ext_B0.y = v0[1]; s->ext_B0.z = v0[2]; }
        s->ext_B_fn = fn; s->ext_B_data = data;
    } else {
        s->ext_E_type = type; s->Ep = s->Epbuf + 1 + s->nrow;
        if (v0) { s->ext_E0.x = v0[0]; s->ext_E0.y = v0[1]; s->ext_E0.z = v0[2]; }
        s->ext_E_fn = fn; s->ext_E_data = data;
    }
    return 0;
}

int zo_sim_set_ext_fld(zo_sim *s, int E_type, const float E0[3], zo_field_fn E_fn, void *E_data,
                       int B_type, const float B0[3], zo_field_fn B_fn, void *B_data)   /* emf.c:764-831 */
{
    if (set_part_grid(s, 0, E_type, E0, E_fn, E_data)) return -1;
    if (set_part_grid(s, 1, B_type, B0, B_fn, B_data)) return -1;
    emf_particle_fields(s);
    return 0;
}

int zo_sim_init_fld(zo_sim *s, int E_type, const float E0[3], zo_field_fn E_fn, void *E_data,
                    int B_type, const float B0[3], zo_field_fn B_fn, void *B_data)      /* emf.c:922-980 */
{
    if (s->emf_iter != 0) return -1;
    const int nrow = s->nrow;
    for (int pass = 0; pass < 2; pass++) {
        const int type = pass ? B_type : E_type;
        if (type == ZO_FLD_NONE) continue;
        zo_f3 *F = pass ? s->B : s->E;
        for (int j = -1; j < s->nx[1] + 2; j++)
            for (int i = -1; i < s->nx[0] + 2; i++) {
                zo_f3 v;
                if (type == ZO_FLD_UNIFORM) {
                    const float *u = pass ? B0 : E0;
                    v.x = u[0]; v.y = u[1]; v.z = u[2];
                } else {
                    float o[3];
                    if (pass) B_fn(i, s->dx[0], j, s->dx[1], B_data, o);
                    else E_fn(i, s->dx[0], j, s->dx[1], E_data, o);
                    v.x = o[0]; v.y = o[1]; v.z = o[2];
                }
                F[j * nrow + i] = v;
            }
    }
    return 0;
}

void zo_sim_iter(zo_sim *s)                                                /* simulation.c:45-56 */
{
    zo_current_zero(s);
    for (int k = 0; k < s->nspec; k++) zo_spec_advance(s, k);
    zo_current_update(s);
    zo_emf_advance(s);
}

/* ---- accessors ---- */
int zo_nrow(const zo_sim *s) { return s->nrow; }
int zo_buf_cells(const zo_sim *s) { return s->ncell_buf; }
int zo_n_species(const zo_sim *s) { return s->nspec; }
int zo_spec_np(const zo_sim *s, int k) { return s->spec[k].np; }
float zo_spec_q(const zo_sim *s, int k) { return s->spec[k].q; }
double zo_spec_energy(const zo_sim *s, int k) { return s->spec[k].energy; }
int zo_spec_n_move(const zo_sim *s, int k) { return s->spec[k].n_move; }
int zo_emf_n_move(const zo_sim *s) { return s->emf_n_move; }
int zo_emf_iter(const zo_sim *s) { return s->emf_iter; }

void zo_get_particles(const zo_sim *s, int k, zo_part *out)
{
    memcpy(out, s->spec[k].p, (size_t)s->spec[k].np * sizeof(zo_part));
}

void zo_set_particles(zo_sim *s, int k, const zo_part *in, int np)
{
    zo_spec *sp = &s->spec[k];
    spec_reserve(sp, np);
    memcpy(sp->p, in, (size_t)np * sizeof(zo_part));
    sp->np = np;
}

void zo_get_E(const zo_sim *s, float *b) { memcpy(b, s->Ebuf, (size_t)s->ncell_buf * sizeof(zo_f3)); }
void zo_get_B(const zo_sim *s, float *b) { memcpy(b, s->Bbuf, (size_t)s->ncell_buf * sizeof(zo_f3)); }
void zo_get_J(const zo_sim *s, float *b) { memcpy(b, s->Jbuf, (size_t)s->ncell_buf * sizeof(zo_f3)); }
void zo_get_E_part(const zo_sim *s, float *b)
{
    memcpy(b, s->Ep - 1 - s->nrow, (size_t)s->ncell_buf * sizeof(zo_f3));
}
void zo_get_B_part(const zo_sim *s, float *b)
{
    memcpy(b, s->Bp - 1 - s->nrow, (size_t)s->ncell_buf * sizeof(zo_f3));
}
void zo_set_E(zo_sim *s, const float *b) { memcpy(s->Ebuf, b, (size_t)s->ncell_buf * sizeof(zo_f3)); }
void zo_set_B(zo_sim *s, const float *b) { memcpy(s->Bbuf, b, (size_t)s->ncell_buf * sizeof(zo_f3)); }
void zo_set_J(zo_sim *s, const float *b) { memcpy(s->Jbuf, b, (size_t)s->ncell_buf * sizeof(zo_f3)); }

void zo_spec_charge(const zo_sim *s, int k, float *rho)                    /* particles.c:1289-1324 */
{
    const zo_spec *sp = &s->spec[k];
    const int nrow = sp->nx[0] + 1;
    const float q = sp->q;
    for (int n = 0; n < sp->np; n++) {
        const int c = sp->p[n].ix + nrow * sp->p[n].iy;
        const float w1 = sp->p[n].x, w2 = sp->p[n].y;
        rho[c] += (1.0f - w1) * (1.0f - w2) * q;
        rho[c + 1] += (w1) * (1.0f - w2) * q;
        rho[c + nrow] += (1.0f - w1) * (w2) * q;
        rho[c + 1 + nrow] += (w1) * (w2) * q;
    }
    if (!sp->moving_window)
        for (int j = 0; j < sp->nx[1] + 1; j++) rho[j * nrow] += rho[sp->nx[0] + j * nrow];
    for (int i = 0; i < sp->nx[0] + 1; i++) rho[i] += rho[i + sp->nx[1] * nrow];
}

/* phase-space density (spec_deposit_pha, particles.c:1569-1632) with the
 * axis quantities of spec_pha_axis (particles.c:1510-1536): quantity codes
 * 1 x1, 2 x2, 4 u1, 5 u2, 6 u3; range = {x1min, x1max, x2min, x2max} */
static float zo_pha_quant(const zo_spec *sp, int n, int q)
{
    switch (q) {
    case 1: return (sp->p[n].x + sp->p[n].ix) * sp->dx[0];
    case 2: return (sp->p[n].y + sp->p[n].iy) * sp->dx[1];
    case 4: return sp->p[n].ux;
    case 5: return sp->p[n].uy;
    default: return sp->p[n].uz;
    }
}

void zo_spec_pha(const zo_sim *s, int k, int q1, int q2, const int pha_nx[2], const float range[4], float *buf)
{
    const zo_spec *sp = &s->spec[k];
    const int nrow = pha_nx[0];
    const float x1min = range[0], x2min = range[2];
    const float rdx1 = pha_nx[0] / (range[1] - range[0]);
    const float rdx2 = pha_nx[1] / (range[3] - range[2]);
    for (int n = 0; n < sp->np; n++) {
        const float nx1 = (zo_pha_quant(sp, n, q1) - x1min) * rdx1;
        const float nx2 = (zo_pha_quant(sp, n, q2) - x2min) * rdx2;
        const int i1 = (int)(nx1 + 0.5f), i2 = (int)(nx2 + 0.5f);
        const float w1 = nx1 - i1 + 0.5f, w2 = nx2 - i2 + 0.5f;
        int idx = i1 + nrow * i2;
        if (i2 >= 0 && i2 < pha_nx[1]) {
            if (i1 >= 0 && i1 < pha_nx[0]) buf[idx] += (1.0f - w1) * (1.0f - w2) * sp->q;
            if (i1 + 1 >= 0 && i1 + 1 < pha_nx[0]) buf[idx + 1] += w1 * (1.0f - w2) * sp->q;
        }
        idx += nrow;
        if (i2 + 1 >= 0 && i2 + 1 < pha_nx[1]) {
            if (i1 >= 0 && i1 < pha_nx[0]) buf[idx] += (1.0f - w1) * w2 * sp->q;
            if (i1 + 1 >= 0 && i1 + 1 < pha_nx[0]) buf[idx + 1] += w1 * w2 * sp->q;
        }
    }
}

