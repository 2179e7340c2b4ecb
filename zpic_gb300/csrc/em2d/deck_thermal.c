/* The uniform thermal plasma workload as a reference input deck run through
 * the em2d drop-in API (include/em2d, libzpic_em2d): one electron species,
 * 4 x 4 particles per cell, uth = 0.05 in every direction, compensated
 * level-1 current smoothing along x and y, dt = 0.05 on a 2048 x 2048 grid
 * of cell size 0.1 (the grid size is an argument).  The main loop is the
 * reference's (em2d/main.c:38-71: sim_iter each step, no reports), timed
 * with the API's own wall clock.
 *
 *   deck_thermal STEPS MIRRORS [NX] [TILE_X TILE_Y FAST]
 *
 * MIRRORS is "every" (the host structs kept valid across every sim_iter, as
 * the reference's callers read them) or "demand" (refreshed by
 * sim_sync_host only).  Prints one "key value" pair per line: the setup
 * time (spec_new on the host, sim_new with the upload), the particle
 * count, the time of the first step and of the rest, and of one
 * sim_sync_host after them. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "simulation.h"
#include "timer.h"

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s STEPS every|demand [NX] [TILE_X TILE_Y FAST]\n", argv[0]);
        return 2;
    }
    const int steps = atoi(argv[1]);
    const int every = strcmp(argv[2], "every") == 0;
    if (steps < 2 || (!every && strcmp(argv[2], "demand") != 0)) {
        fprintf(stderr, "STEPS must be >= 2 and MIRRORS every or demand\n");
        return 2;
    }
    const int n = argc > 3 ? atoi(argv[3]) : 2048;
    if (n < 16) {
        fprintf(stderr, "NX must be >= 16\n");
        return 2;
    }
    if (argc > 6) sim_set_gpu_options(0, atoi(argv[4]), atoi(argv[5]), atoi(argv[6]));

    int nx[2] = {n, n};
    float box[2] = {0.1f * n, 0.1f * n};
    const float dt = 0.05f;
    int ppc[2] = {4, 4};
    float ufl[3] = {0.0f, 0.0f, 0.0f};
    float uth[3] = {0.05f, 0.05f, 0.05f};

    const uint64_t t0 = timer_ticks();
    t_species *species = (t_species *)malloc(sizeof(t_species));
    spec_new(&species[0], "electrons", -1.0f, ppc, ufl, uth, nx, box, dt, NULL);
    t_simulation sim;
    sim_new(&sim, nx, box, dt, steps * dt, 0, species, 1);
    t_smooth smooth = {.xtype = COMPENSATED, .ytype = COMPENSATED, .xlevel = 1, .ylevel = 1};
    sim_set_smooth(&sim, &smooth);
    sim_set_mirrors(&sim, every);
    const uint64_t t1 = timer_ticks();

    sim_iter(&sim);
    const uint64_t t2 = timer_ticks();
    for (int i = 1; i < steps; i++) sim_iter(&sim);
    const uint64_t t3 = timer_ticks();

    /* one full host refresh (what a report or a direct reader pays) */
    const uint64_t t4 = timer_ticks();
    sim_sync_host(&sim);
    const uint64_t t5 = timer_ticks();
    double emf[6];
    emf_get_energy(&sim.emf, emf);
    printf("setup_s %.6f\n", timer_interval_seconds(t0, t1));
    printf("particles %d\n", sim.species[0].np);
    printf("first_step_ms %.6f\n", 1e3 * timer_interval_seconds(t1, t2));
    printf("step_ms %.6f\n", 1e3 * timer_interval_seconds(t2, t3) / (steps - 1));
    printf("sync_host_ms %.6f\n", 1e3 * timer_interval_seconds(t4, t5));
    printf("kinetic %.17g\n", sim.species[0].energy);
    printf("field %.17g\n", emf[0] + emf[1] + emf[2] + emf[3] + emf[4] + emf[5]);
    sim_delete(&sim);
    return 0;
}
