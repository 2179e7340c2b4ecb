/*
 * zpic_oracle_em1d.c -- CPU restatement of the reference's em1d time step,
 * the checker of the 1-D GPU step (zc1_*) and, built with the reference's
 * stock -Ofast flags, its timed CPU baseline where the reference itself is
 * not built.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, the smoke check and bench.py's CPU
 * baseline load it; the product never does.
 *
 * It exports the checker ABI of ref_driver_em1d.c (prefix zr1_), so that
 * oracle/pyoracle_em1d.RefSim1D runs on either library.  Plain loops over
 * float3 buffers of nx + 3 cells (one lower, two upper guard cells), in the
 * reference's order of operations: a strict IEEE build (-ffp-contract=off)
 * gives the reference's bits (pinned by tests/test_em1d.py against the
 * fixtures the reference made).
 *
 *   sim_iter            em1d/simulation.c:45-56
 *   spec_new, loading   em1d/particles.c:72-135 (spec_set_u), 250-447
 *                       (spec_set_x: uniform, empty, step, slab), 475-589
 *   spec_advance        em1d/particles.c:864-894 (interpolate_fld), 707-790
 *                       (dep_current_zamb), 923-1070 (Boris, push,
 *                       boundaries, window, sort)
 *   spec_sort           em1d/particles.c:796-843 (a stable counting sort)
 *   current_update      em1d/current.c:93-156, 244-330
 *   emf_advance         em1d/emf.c:379-415 (Mur), 422-460 (Yee), 470-566
 *   emf_add_laser       em1d/emf.c:157-260
 *   emf_get_energy      em1d/emf.c:590-612
 *   rand_norm           em1d/random.c (the MWC generator and polar
 *                       Box-Muller; set_rand_seed keeps the cached deviate,
 *                       as the reference does)
 *
 * Ramp and custom density profiles and external fields are not restated
 * (the GPU step takes neither).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } f3;
typedef struct { int ix; float x, ux, uy, uz; } zr1_part;

enum { D_UNIFORM = 0, D_EMPTY = 1, D_STEP = 2, D_SLAB = 3 };
enum { BC_NONE = 0, BC_PERIODIC = 1, BC_OPEN = 2 };

/* ------------------------------------------------------------------ random */
static uint32_t m_w = 12345, m_z = 67890;
static int rn_iset = 0;
static double rn_gset = 0.0;

void zr1_set_rand_seed(uint32_t w, uint32_t z)
{
    m_w = w;
    m_z = z;
}

static uint32_t rand_u32(void)
{
    m_z = 36969 * (m_z & 65535) + (m_z >> 16);
    m_w = 18000 * (m_w & 65535) + (m_w >> 16);
    return (m_z << 16) + m_w;
}

static double rand_norm(void)
{
    if (rn_iset) {
        rn_iset = 0;
        return rn_gset;
    }
    double v1, v2, rsq;
    do {
        v1 = (rand_u32() + 0.5) / 2147483649.0 - 1.0;
        v2 = (rand_u32() + 0.5) / 2147483649.0 - 1.0;
        rsq = v1 * v1 + v2 * v2;
    } while (rsq == 0.0 || rsq >= 1.0);
    const double fac = sqrt(-2.0 * log(rsq) / rsq);
    rn_gset = v1 * fac;
    rn_iset = 1;
    return v2 * fac;
}

/* --------------------------------------------------------------- structures */
typedef struct {
    float m_q, q;
    int ppc;
    float ufl[3], uth[3];
    int dtype;
    float dstart, dend;
    zr1_part *part;
    int np, np_max;
    int iter, n_move, moving_window, n_sort, open;
    double energy;
} spec1;

typedef struct {
    int nx;
    float box, dx, dt;
    spec1 *spec;
    int nspec;
    f3 *Ebuf, *Bbuf, *Jbuf;     /* cell i at buf[i + 1] */
    int emf_bc, cur_bc;
    int emf_iter, n_move, moving_window;
    f3 mur_fld[2], mur_tmp[2];
    int smooth_type, smooth_level;
} zr1_sim;

#define CELL(buf, i) ((buf)[(i) + 1])

zr1_sim *zr1_sim_new(int nx, float box, float dt)
{
    zr1_sim *s = (zr1_sim *)calloc(1, sizeof(zr1_sim));
    s->nx = nx;
    s->box = box;
    s->dx = box / nx;
    s->dt = dt;
    return s;
}

/* ------------------------------------------------------------------ loading */
static void grow(spec1 *p, int size)
{
    if (size > p->np_max) {
        p->np_max = (size / 1024 + 1) * 1024;
        p->part = (zr1_part *)realloc(p->part, (size_t)p->np_max * sizeof(zr1_part));
    }
}

/* positions of the new particles in cells [i0, i1] (spec_set_x) */
static void set_x(spec1 *p, float dx, int i0, int i1)
{
    const int npc = p->ppc;
    float *poscell = (float *)malloc(sizeof(float) * (size_t)npc);
    for (int k = 0; k < npc; k++) poscell[k] = (k + 0.5) / npc;
    grow(p, p->np + (i1 - i0 + 1) * npc);
    int ip = p->np;
    if (p->dtype == D_STEP) {
        const float start = p->dstart / dx - p->n_move;
        for (int i = i0; i <= i1; i++)
            for (int k = 0; k < npc; k++)
                if (i + poscell[k] > start) {
                    p->part[ip].ix = i;
                    p->part[ip].x = poscell[k];
                    ip++;
                }
    } else if (p->dtype == D_SLAB) {
        const float start = p->dstart / dx - p->n_move;
        const float end = p->dend / dx - p->n_move;
        for (int i = i0; i <= i1; i++)
            for (int k = 0; k < npc; k++)
                if (i + poscell[k] > start && i + poscell[k] < end) {
                    p->part[ip].ix = i;
                    p->part[ip].x = poscell[k];
                    ip++;
                }
    } else if (p->dtype == D_UNIFORM) {
        for (int i = i0; i <= i1; i++)
            for (int k = 0; k < npc; k++) {
                p->part[ip].ix = i;
                p->part[ip].x = poscell[k];
                ip++;
            }
    }
    free(poscell);
    p->np = ip;
}

/* thermal momenta, per-cell mean removed, plus the fluid momentum (spec_set_u) */
static void set_u(spec1 *p, int nx, int start, int end)
{
    for (int i = start; i <= end; i++) {
        p->part[i].ux = p->uth[0] * rand_norm();
        p->part[i].uy = p->uth[1] * rand_norm();
        p->part[i].uz = p->uth[2] * rand_norm();
    }
    f3 *net = (f3 *)calloc((size_t)nx, sizeof(f3));
    int *cnt = (int *)calloc((size_t)nx, sizeof(int));
    for (int i = start; i <= end; i++) {
        const int c = p->part[i].ix;
        net[c].x += p->part[i].ux;
        net[c].y += p->part[i].uy;
        net[c].z += p->part[i].uz;
        cnt[c] += 1;
    }
    for (int c = 0; c < nx; c++) {
        const float norm = (cnt[c] > 0) ? 1.0f / cnt[c] : 0;
        net[c].x *= norm;
        net[c].y *= norm;
        net[c].z *= norm;
    }
    for (int i = start; i <= end; i++) {
        const int c = p->part[i].ix;
        p->part[i].ux += p->ufl[0] - net[c].x;
        p->part[i].uy += p->ufl[1] - net[c].y;
        p->part[i].uz += p->ufl[2] - net[c].z;
    }
    free(cnt);
    free(net);
}

static void inject(spec1 *p, int nx, float dx, int i0, int i1)
{
    const int start = p->np;
    set_x(p, dx, i0, i1);
    set_u(p, nx, start, p->np - 1);
}

/* density type: UNIFORM 0, EMPTY 1, STEP 2, SLAB 3 (density n scales q) */
int zr1_add_species(zr1_sim *s, const char *name, float m_q, int ppc, const float ufl[3], const float uth[3],
                    int dtype, float start, float end, float n)
{
    (void)name;
    s->spec = (spec1 *)realloc(s->spec, (size_t)(s->nspec + 1) * sizeof(spec1));
    spec1 *p = &s->spec[s->nspec];
    memset(p, 0, sizeof(*p));
    p->m_q = m_q;
    p->ppc = ppc;
    p->q = copysign(1.0f, m_q) / ppc;  /* in double, then rounded (particles.c:529) */
    if (n == 0.f) n = 1.0f;
    p->q *= fabsf(n);
    for (int i = 0; i < 3; i++) {
        p->ufl[i] = ufl ? ufl[i] : 0.f;
        p->uth[i] = uth ? uth[i] : 0.f;
    }
    p->dtype = dtype;
    p->dstart = start;
    p->dend = end;
    inject(p, s->nx, s->dx, 0, s->nx - 1);
    p->n_sort = 16;
    return s->nspec++;
}

void zr1_finalize(zr1_sim *s)
{
    const size_t n = (size_t)s->nx + 3;
    s->Ebuf = (f3 *)calloc(n, sizeof(f3));
    s->Bbuf = (f3 *)calloc(n, sizeof(f3));
    s->Jbuf = (f3 *)calloc(n, sizeof(f3));
    s->emf_bc = BC_PERIODIC;
    s->cur_bc = BC_PERIODIC;
}

void zr1_sim_delete(zr1_sim *s)
{
    for (int k = 0; k < s->nspec; k++) free(s->spec[k].part);
    free(s->spec);
    free(s->Ebuf);
    free(s->Bbuf);
    free(s->Jbuf);
    free(s);
}

void zr1_set_smooth(zr1_sim *s, int type, int level)
{
    s->smooth_type = type;
    s->smooth_level = level;
}

void zr1_set_moving_window(zr1_sim *s)
{
    s->moving_window = 1;
    s->emf_bc = BC_NONE;
    s->cur_bc = BC_NONE;
    for (int k = 0; k < s->nspec; k++) s->spec[k].moving_window = 1;
}

void zr1_set_open(zr1_sim *s, int fields, int particles)
{
    if (fields) s->emf_bc = BC_OPEN;
    if (particles)
        for (int k = 0; k < s->nspec; k++) s->spec[k].open = 1;
}

void zr1_set_n_sort(zr1_sim *s, int k, int n) { s->spec[k].n_sort = n; }

/* -------------------------------------------------------------------- fields */
static void emf_gc(zr1_sim *s)
{
    if (s->emf_bc != BC_PERIODIC) return;
    const int nx = s->nx;
    CELL(s->Ebuf, -1) = CELL(s->Ebuf, nx - 1);
    CELL(s->Bbuf, -1) = CELL(s->Bbuf, nx - 1);
    CELL(s->Ebuf, nx) = CELL(s->Ebuf, 0);
    CELL(s->Bbuf, nx) = CELL(s->Bbuf, 0);
}

static float lon_env(float start, float rise, float flat, float fall, float z)
{
    if (z > start) return 0.0f;
    if (z > start - rise) {
        const float csi = z - start;
        const float e = sin(M_PI_2 * csi / rise);
        return e * e;
    }
    if (z > start - (rise + flat)) return 1.0f;
    if (z > start - (rise + flat + fall)) {
        const float csi = z - (start - rise - flat - fall);
        const float e = sin(M_PI_2 * csi / fall);
        return e * e;
    }
    return 0.0f;
}

void zr1_add_laser(zr1_sim *s, float start, float fwhm, float a0, float omega0, float polarization)
{
    /* the fwhm form (rise = fall = fwhm, no flat top) */
    const float rise = fwhm, fall = fwhm, flat = 0.f;
    f3 *E = s->Ebuf + 1, *B = s->Bbuf + 1;
    const float dx = s->dx;
    const float amp = omega0 * a0;
    const float cos_pol = cos(polarization), sin_pol = sin(polarization);
    const float k = omega0;
    for (int i = 0; i < s->nx; i++) {
        const float z = i * dx;
        const float z_2 = z + dx / 2;
        const float lenv = amp * lon_env(start, rise, flat, fall, z);
        const float lenv_2 = amp * lon_env(start, rise, flat, fall, z_2);
        E[i].y += +lenv * cos(k * z) * cos_pol;
        E[i].z += +lenv * cos(k * z) * sin_pol;
        B[i].y += -lenv_2 * cos(k * z_2) * sin_pol;
        B[i].z += +lenv_2 * cos(k * z_2) * cos_pol;
    }
    emf_gc(s);
}

static void yee_b(zr1_sim *s, float dt)
{
    f3 *restrict B = s->Bbuf + 1;
    const f3 *restrict E = s->Ebuf + 1;
    const float dt_dx = dt / s->dx;
    for (int i = -1; i <= s->nx; i++) {
        B[i].y += (dt_dx * (E[i + 1].z - E[i].z));
        B[i].z += (-dt_dx * (E[i + 1].y - E[i].y));
    }
}

static void yee_e(zr1_sim *s, float dt)
{
    f3 *restrict E = s->Ebuf + 1;
    const f3 *restrict B = s->Bbuf + 1;
    const f3 *restrict J = s->Jbuf + 1;
    const float dt_dx = dt / s->dx;
    for (int i = 0; i <= s->nx + 1; i++) {
        E[i].x += (-dt * J[i].x);
        E[i].y += (-dt_dx * (B[i].z - B[i - 1].z) - dt * J[i].y);
        E[i].z += (+dt_dx * (B[i].y - B[i - 1].y) - dt * J[i].z);
    }
}

static void mur(zr1_sim *s)
{
    f3 *E = s->Ebuf + 1;
    const int nx = s->nx;
    const float S = (s->dt - s->dx) / (s->dt + s->dx);
    s->mur_fld[0].y = s->mur_tmp[0].y + S * (E[0].y - s->mur_fld[0].y);
    s->mur_fld[0].z = s->mur_tmp[0].z + S * (E[0].z - s->mur_fld[0].z);
    E[-1].y = s->mur_fld[0].y;
    E[-1].z = s->mur_fld[0].z;
    s->mur_tmp[0].y = E[0].y;
    s->mur_tmp[0].z = E[0].z;
    s->mur_fld[1].y = s->mur_tmp[1].y + S * (E[nx - 1].y - s->mur_fld[1].y);
    s->mur_fld[1].z = s->mur_tmp[1].z + S * (E[nx - 1].z - s->mur_fld[1].z);
    E[nx].y = s->mur_fld[1].y;
    E[nx].z = s->mur_fld[1].z;
    s->mur_tmp[1].y = E[nx - 1].y;
    s->mur_tmp[1].z = E[nx - 1].z;
}

static void emf_advance(zr1_sim *s)
{
    const float dt = s->dt;
    yee_b(s, dt / 2.0f);
    yee_e(s, dt);
    if (s->emf_bc == BC_OPEN) mur(s);
    yee_b(s, dt / 2.0f);
    emf_gc(s);
    s->emf_iter += 1;
    if (s->moving_window && (s->emf_iter * s->dt) > s->dx * (s->n_move + 1)) {
        f3 *E = s->Ebuf + 1, *B = s->Bbuf + 1;
        for (int i = -1; i < s->nx + 2 - 1; i++) {
            E[i] = E[i + 1];
            B[i] = B[i + 1];
        }
        const f3 zero = {0.f, 0.f, 0.f};
        for (int i = s->nx - 1; i < s->nx + 2; i++) {
            E[i] = zero;
            B[i] = zero;
        }
        s->n_move++;
    }
}

void zr1_emf_energy(const zr1_sim *s, double en[6])
{
    const f3 *E = s->Ebuf + 1, *B = s->Bbuf + 1;
    for (int c = 0; c < 6; c++) en[c] = 0;
    for (int i = 0; i < s->nx; i++) {
        en[0] += E[i].x * E[i].x;
        en[1] += E[i].y * E[i].y;
        en[2] += E[i].z * E[i].z;
        en[3] += B[i].x * B[i].x;
        en[4] += B[i].y * B[i].y;
        en[5] += B[i].z * B[i].z;
    }
    for (int c = 0; c < 6; c++) en[c] *= 0.5 * s->dx;
}

/* ------------------------------------------------------------------- current */
static void kernel_x(zr1_sim *s, float sa, float sb)
{
    f3 *restrict J = s->Jbuf + 1;
    f3 fl = J[-1], f0 = J[0];
    for (int i = 0; i < s->nx; i++) {
        const f3 fu = J[i + 1];
        f3 fs;
        fs.x = sa * fl.x + sb * f0.x + sa * fu.x;
        fs.y = sa * fl.y + sb * f0.y + sa * fu.y;
        fs.z = sa * fl.z + sb * f0.z + sa * fu.z;
        J[i] = fs;
        fl = f0;
        f0 = fu;
    }
    if (s->cur_bc == BC_PERIODIC) {
        J[-1] = J[s->nx - 1];
        for (int i = 0; i < 2; i++) J[s->nx + i] = J[i];
    }
}

static void current_update(zr1_sim *s)
{
    f3 *restrict J = s->Jbuf + 1;
    const int nx = s->nx;
    if (s->cur_bc == BC_PERIODIC) {
        for (int i = -1; i < 2; i++) {
            J[i].x += J[nx + i].x;
            J[i].y += J[nx + i].y;
            J[i].z += J[nx + i].z;
        }
        for (int i = -1; i < 2; i++) J[nx + i] = J[i];
    }
    if (s->smooth_type != 0) {
        for (int i = 0; i < s->smooth_level; i++) kernel_x(s, 0.25, 0.5);
        if (s->smooth_type == 2) {
            const int n = s->smooth_level;
            const float a = -1;
            const float b = (4.0 + 2.0 * n) / n;
            const float total = 2 * a + b;
            kernel_x(s, a / total, b / total);
        }
    }
}

/* ----------------------------------------------------------------- particles */
static void dep_zamb(f3 *restrict J, int ix0, int di, float x0, float dx, float qnx, float qvy, float qvz)
{
    struct { float x0, x1, dx, qvy, qvz; int ix; } vp[2];
    int vnp = 1;
    vp[0].x0 = x0;
    vp[0].dx = dx;
    vp[0].x1 = x0 + dx;
    vp[0].qvy = qvy / 2.0;
    vp[0].qvz = qvz / 2.0;
    vp[0].ix = ix0;
    if (di != 0) {
        const int ib = (di == 1);
        const float delta = (x0 + dx - ib) / dx;
        vp[1].x0 = 1 - ib;
        vp[1].x1 = (x0 + dx) - di;
        vp[1].dx = dx * delta;
        vp[1].ix = ix0 + di;
        vp[1].qvy = vp[0].qvy * delta;
        vp[1].qvz = vp[0].qvz * delta;
        vp[0].x1 = ib;
        vp[0].dx *= (1.0f - delta);
        vp[0].qvy *= (1.0f - delta);
        vp[0].qvz *= (1.0f - delta);
        vnp++;
    }
    for (int k = 0; k < vnp; k++) {
        const float s00 = 1.0f - vp[k].x0, s01 = vp[k].x0;
        const float s10 = 1.0f - vp[k].x1, s11 = vp[k].x1;
        J[vp[k].ix].x += qnx * vp[k].dx;
        J[vp[k].ix].y += vp[k].qvy * (s00 + s10 + (s00 - s10) / 2.0f);
        J[vp[k].ix + 1].y += vp[k].qvy * (s01 + s11 + (s01 - s11) / 2.0f);
        J[vp[k].ix].z += vp[k].qvz * (s00 + s10 + (s00 - s10) / 2.0f);
        J[vp[k].ix + 1].z += vp[k].qvz * (s01 + s11 + (s01 - s11) / 2.0f);
    }
}

/* stable counting sort by cell: the order the reference's in-place
 * permutation of spec_sort leaves */
static void sort_cells(spec1 *p, int nx)
{
    int *cnt = (int *)calloc((size_t)nx + 1, sizeof(int));
    zr1_part *out = (zr1_part *)malloc(sizeof(zr1_part) * (size_t)(p->np > 0 ? p->np : 1));
    for (int i = 0; i < p->np; i++) cnt[p->part[i].ix + 1]++;
    for (int c = 0; c < nx; c++) cnt[c + 1] += cnt[c];
    for (int i = 0; i < p->np; i++) out[cnt[p->part[i].ix]++] = p->part[i];
    memcpy(p->part, out, sizeof(zr1_part) * (size_t)p->np);
    free(out);
    free(cnt);
}

static void spec_advance(zr1_sim *s, spec1 *p)
{
    const float tem = 0.5 * s->dt / p->m_q;
    const float dt_dx = s->dt / s->dx;
    const float qnx = p->q * s->dx / s->dt;
    const int nx0 = s->nx;
    const f3 *restrict E = s->Ebuf + 1;
    const f3 *restrict B = s->Bbuf + 1;
    f3 *restrict J = s->Jbuf + 1;
    double energy = 0;
    for (int i = 0; i < p->np; i++) {
        zr1_part *pt = &p->part[i];
        float ux = pt->ux, uy = pt->uy, uz = pt->uz;
        /* interpolate_fld */
        const int ic = pt->ix;
        const float w1 = pt->x;
        const int ih = ic + ((w1 < 0.5f) ? -1 : 0);
        const float w1h = w1 + ((w1 < 0.5f) ? 0.5f : -0.5f);
        f3 Ep, Bp;
        Ep.x = E[ih].x * (1.0f - w1h) + E[ih + 1].x * w1h;
        Ep.y = E[ic].y * (1.0f - w1) + E[ic + 1].y * w1;
        Ep.z = E[ic].z * (1.0f - w1) + E[ic + 1].z * w1;
        Bp.x = B[ic].x * (1.0f - w1) + B[ic + 1].x * w1;
        Bp.y = B[ih].y * (1.0f - w1h) + B[ih + 1].y * w1h;
        Bp.z = B[ih].z * (1.0f - w1h) + B[ih + 1].z * w1h;
        /* Boris */
        Ep.x *= tem;
        Ep.y *= tem;
        Ep.z *= tem;
        float utx = ux + Ep.x, uty = uy + Ep.y, utz = uz + Ep.z;
        const float u2 = utx * utx + uty * uty + utz * utz;
        const float gamma = sqrtf(1 + u2);
        energy += u2 / (1 + gamma);
        const float gtem = tem / gamma;
        Bp.x *= gtem;
        Bp.y *= gtem;
        Bp.z *= gtem;
        const float otsq = 2.0f / (1.0f + Bp.x * Bp.x + Bp.y * Bp.y + Bp.z * Bp.z);
        ux = utx + uty * Bp.z - utz * Bp.y;
        uy = uty + utz * Bp.x - utx * Bp.z;
        uz = utz + utx * Bp.y - uty * Bp.x;
        Bp.x *= otsq;
        Bp.y *= otsq;
        Bp.z *= otsq;
        utx += uy * Bp.z - uz * Bp.y;
        uty += uz * Bp.x - ux * Bp.z;
        utz += ux * Bp.y - uy * Bp.x;
        ux = utx + Ep.x;
        uy = uty + Ep.y;
        uz = utz + Ep.z;
        pt->ux = ux;
        pt->uy = uy;
        pt->uz = uz;
        /* push and deposit */
        const float rg = 1.0f / sqrtf(1.0f + ux * ux + uy * uy + uz * uz);
        const float dx = dt_dx * rg * ux;
        float x1 = pt->x + dx;
        const int di = (x1 >= 1.0f) - (x1 < 0.0f);
        x1 -= di;
        const float qvy = p->q * uy * rg;
        const float qvz = p->q * uz * rg;
        dep_zamb(J, pt->ix, di, pt->x, dx, qnx, qvy, qvz);
        pt->x = x1;
        pt->ix += di;
    }
    p->energy = p->q * p->m_q * energy * s->dx;
    p->iter += 1;
    if (p->moving_window || p->open) {
        if (p->moving_window && (p->iter * s->dt) > (s->dx * (p->n_move + 1))) {
            for (int i = 0; i < p->np; i++) p->part[i].ix--;
            p->n_move++;
            inject(p, s->nx, s->dx, s->nx - 1, s->nx - 1);
        }
        int i = 0;
        while (i < p->np) {
            if (p->part[i].ix < 0 || p->part[i].ix >= nx0) {
                p->part[i] = p->part[--p->np];
                continue;
            }
            i++;
        }
    } else {
        for (int i = 0; i < p->np; i++)
            p->part[i].ix += ((p->part[i].ix < 0) ? nx0 : 0) - ((p->part[i].ix >= nx0) ? nx0 : 0);
    }
    if (p->n_sort > 0 && !(p->iter % p->n_sort)) sort_cells(p, s->nx);
}

/* ---------------------------------------------------------------- the step */
void zr1_iter(zr1_sim *s)
{
    memset(s->Jbuf, 0, ((size_t)s->nx + 3) * sizeof(f3));
    for (int k = 0; k < s->nspec; k++) spec_advance(s, &s->spec[k]);
    current_update(s);
    emf_advance(s);
}

int zr1_spec_np(const zr1_sim *s, int k) { return s->spec[k].np; }
float zr1_spec_q(const zr1_sim *s, int k) { return s->spec[k].q; }
double zr1_spec_energy(const zr1_sim *s, int k) { return s->spec[k].energy; }
int zr1_n_move(const zr1_sim *s) { return s->n_move; }

void zr1_get_particles(const zr1_sim *s, int k, zr1_part *out)
{
    memcpy(out, s->spec[k].part, (size_t)s->spec[k].np * sizeof(zr1_part));
}

static size_t nbytes(const zr1_sim *s) { return ((size_t)s->nx + 3) * sizeof(f3); }
void zr1_get_E(const zr1_sim *s, float *b) { memcpy(b, s->Ebuf, nbytes(s)); }
void zr1_get_B(const zr1_sim *s, float *b) { memcpy(b, s->Bbuf, nbytes(s)); }
void zr1_get_J(const zr1_sim *s, float *b) { memcpy(b, s->Jbuf, nbytes(s)); }
