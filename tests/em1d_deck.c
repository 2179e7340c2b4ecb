/*
 * em1d_deck.c -- a deck program written against the em1d C API only
 * (sim_new, spec_new, sim_iter, the reports).  The tests build it twice:
 * against the reference's em1d sources (tests/golden/make_em1d_reports.py,
 * which writes the golden report files) and against the drop-in headers and
 * libzpic_em1d (tests/test_em1d_dropin.py), and compare the report files.
 *
 *     em1d_deck <deck> <steps>
 *
 * Decks: "lwfa" (moving window, laser, cold step plasma injected by the
 * window), "twostream" (two periodic drifting streams), "absorbing" (open
 * fields and particles set by writing the struct fields after sim_new, a
 * laser entering a warm slab), "density" (a ramp and a custom profile,
 * compared at loading only).  Reports are written after loading and after
 * the last step, into the working directory.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "simulation.h"

static void setup_lwfa(t_simulation *sim)
{
    const int nx = 300;
    const float box = 6.0f, dt = 0.019f;
    t_species *sp = (t_species *)malloc(sizeof(t_species));
    t_density density;
    memset(&density, 0, sizeof(density));
    density.type = STEP;
    density.start = 6.0f;
    spec_new(&sp[0], "electrons", -1.0f, 16, NULL, NULL, nx, box, dt, &density);
    sim_new(sim, nx, box, dt, 10.0f, 0, sp, 1);
    t_emf_laser laser;
    memset(&laser, 0, sizeof(laser));
    laser.start = 5.0f;
    laser.fwhm = 1.0f;
    laser.a0 = 2.0f;
    laser.omega0 = 10.0f;
    laser.polarization = M_PI_2;
    sim_add_laser(sim, &laser);
    sim_set_moving_window(sim);
    t_smooth smooth = {.xtype = COMPENSATED, .xlevel = 2};
    sim_set_smooth(sim, &smooth);
}

static void setup_twostream(t_simulation *sim)
{
    const int nx = 120;
    const float box = 4 * M_PI, dt = 0.1f;
    t_species *sp = (t_species *)malloc(2 * sizeof(t_species));
    const float ufl_r[] = {0.2f, 0.0f, 0.0f}, ufl_l[] = {-0.1f, 0.05f, 0.03f};
    const float uth[] = {0.001f, 0.001f, 0.001f};
    spec_new(&sp[0], "right", -1.0f, 16, ufl_r, uth, nx, box, dt, NULL);
    spec_new(&sp[1], "left", -1.0f, 16, ufl_l, uth, nx, box, dt, NULL);
    sim_new(sim, nx, box, dt, 10.0f, 0, sp, 2);
    t_smooth smooth = {.xtype = COMPENSATED, .xlevel = 1};
    sim_set_smooth(sim, &smooth);
}

static void setup_absorbing(t_simulation *sim)
{
    const int nx = 300;
    const float box = 6.0f, dt = 0.019f;
    t_species *sp = (t_species *)malloc(sizeof(t_species));
    const float uth[] = {0.02f, 0.02f, 0.02f};
    t_density density;
    memset(&density, 0, sizeof(density));
    density.type = SLAB;
    density.start = 3.0f;
    density.end = 5.0f;
    spec_new(&sp[0], "electrons", -1.0f, 16, NULL, uth, nx, box, dt, &density);
    sim_new(sim, nx, box, dt, 10.0f, 0, sp, 1);
    t_emf_laser laser;
    memset(&laser, 0, sizeof(laser));
    laser.start = 2.5f;
    laser.fwhm = 0.8f;
    laser.a0 = 1.0f;
    laser.omega0 = 10.0f;
    laser.polarization = 0.3f;
    sim_add_laser(sim, &laser);
    /* open boundaries the way the reference's absorbing deck sets them */
    sim->emf.bc_type = EMF_BC_OPEN;
    sp[0].bc_type = PART_BC_OPEN;
    t_smooth smooth = {.xtype = BINOMIAL, .xlevel = 2};
    sim_set_smooth(sim, &smooth);
}

static float custom_profile(float x, void *data)
{
    (void)data;
    return 1.0f + 0.5f * sinf(x / 2.0f) * sinf(x / 2.0f);
}

/* loading only: a linear ramp and a custom profile (periodic, no window) */
static void setup_density(t_simulation *sim)
{
    const int nx = 200;
    const float box = 10.0f, dt = 0.04f;
    t_species *sp = (t_species *)malloc(2 * sizeof(t_species));
    t_density ramp;
    memset(&ramp, 0, sizeof(ramp));
    ramp.type = RAMP;
    ramp.start = 2.0f;
    ramp.end = 8.0f;
    ramp.ramp[0] = 0.5f;
    ramp.ramp[1] = 2.0f;
    spec_new(&sp[0], "ramp", -1.0f, 16, NULL, NULL, nx, box, dt, &ramp);
    t_density custom;
    memset(&custom, 0, sizeof(custom));
    custom.type = CUSTOM;
    custom.custom = &custom_profile;
    const float uth[] = {0.01f, 0.02f, 0.03f};
    spec_new(&sp[1], "custom", -1.0f, 8, NULL, uth, nx, box, dt, &custom);
    sim_new(sim, nx, box, dt, 10.0f, 0, sp, 2);
}

static void reports(t_simulation *sim)
{
    for (int fc = 0; fc < 3; fc++) {
        emf_report(&sim->emf, EFLD, fc);
        emf_report(&sim->emf, BFLD, fc);
        current_report(&sim->current, fc);
    }
    const int pha_nx[] = {64, 32};
    const float pha_range[][2] = {{0.0f, (float)sim->emf.box}, {-0.5f, 0.5f}};
    for (int k = 0; k < sim->n_species; k++) {
        spec_report(&sim->species[k], CHARGE, NULL, NULL);
        spec_report(&sim->species[k], PHASESPACE(X1, U1), pha_nx, pha_range);
        spec_report(&sim->species[k], PARTICLES, NULL, NULL);
    }
    sim_report_energy(sim);
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: em1d_deck <lwfa|twostream|absorbing> <steps>\n");
        return 2;
    }
    t_simulation sim;
    if (!strcmp(argv[1], "lwfa"))
        setup_lwfa(&sim);
    else if (!strcmp(argv[1], "twostream"))
        setup_twostream(&sim);
    else if (!strcmp(argv[1], "absorbing"))
        setup_absorbing(&sim);
    else if (!strcmp(argv[1], "density"))
        setup_density(&sim);
    else if (!strcmp(argv[1], "extfld")) {
        /* external fields: the 1-D GPU step has none, the drop-in stops */
        setup_twostream(&sim);
        t_emf_ext_fld ext;
        memset(&ext, 0, sizeof(ext));
        ext.B_type = EMF_FLD_TYPE_UNIFORM;
        ext.B_0.x = 0.5f;
        sim_set_ext_fld(&sim, &ext);
    }
    else {
        fprintf(stderr, "unknown deck %s\n", argv[1]);
        return 2;
    }
    const int steps = atoi(argv[2]);
    reports(&sim);
    for (int n = 0; n < steps; n++) sim_iter(&sim);
    if (steps > 0) reports(&sim);
    printf("n_move %d\n", sim.emf.n_move);
    sim_delete(&sim);
    return 0;
}
