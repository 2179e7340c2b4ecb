/* A C input deck driven through the em2d drop-in API (include/em2d,
 * libzpic_em2d): two counter-streaming electron species with compensated x
 * and binomial y smoothing -- the weibel_smooth deck of tests/decks.py --
 * stepped N times with sim_iter, then the field energy per component
 * (emf_get_energy) and each species' kinetic energy, one number per line.
 * Written the way a reference deck + main loop uses the API
 * (em2d/main.c, em2d/input/weibel.c). */
#include <stdio.h>
#include <stdlib.h>

#include "simulation.h"

int main(int argc, char **argv)
{
    const int steps = argc > 1 ? atoi(argv[1]) : 10;
    int nx[2] = {32, 24};
    float box[2] = {3.2f, 2.4f};
    const float dt = 0.07f;
    int ppc[2] = {2, 2};
    float ufl_a[3] = {0.0f, 0.0f, 0.6f}, ufl_b[3] = {0.0f, 0.0f, -0.6f};
    float uth[3] = {0.1f, 0.1f, 0.1f};

    /* the simulation owns (and sim_delete frees) the species array */
    t_species *species = (t_species *)malloc(2 * sizeof(t_species));
    spec_new(&species[0], "e1", -1.0f, ppc, ufl_a, uth, nx, box, dt, NULL);
    spec_new(&species[1], "e2", -1.0f, ppc, ufl_b, uth, nx, box, dt, NULL);

    t_simulation sim;
    sim_new(&sim, nx, box, dt, steps * dt, 0, species, 2);
    t_smooth smooth = {.xtype = COMPENSATED, .ytype = BINOMIAL, .xlevel = 2, .ylevel = 1};
    sim_set_smooth(&sim, &smooth);

    for (int n = 0; n < steps; n++) sim_iter(&sim);

    double emf[6];
    emf_get_energy(&sim.emf, emf);
    sim_sync_host(&sim);
    for (int i = 0; i < 6; i++) printf("emf %.17g\n", emf[i]);
    for (int k = 0; k < 2; k++) printf("kin %.17g\n", sim.species[k].energy);
    for (int k = 0; k < 2; k++) printf("np %d\n", sim.species[k].np);
    sim_delete(&sim);
    return 0;
}
