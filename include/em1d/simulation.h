/* simulation.h -- the em1d drop-in API (libzpic_em1d): the reference's em1d
 * simulation interface (em1d/simulation.h) over the 1-D GPU step of
 * libzpic_cuda (zc1_*).  A deck written for the reference (sim_init,
 * sim_report and the main loop of em1d/main.c) compiles against these
 * headers and runs its steps on the GPU.
 *
 * The GPU simulation is created by the first step, from the state the deck
 * has set up by then: boundaries (including direct writes such as
 * emf.bc_type = EMF_BC_OPEN), lasers and initial fields on the host mirrors,
 * loaded particles, smoothing.  Limits of the 1-D GPU step: no external
 * fields; with open particles every species is open; under a moving window
 * the injected species are cold (uth = 0) with uniform, step or slab
 * profiles.
 *
 * The phase calls current_zero, spec_advance and current_update do nothing;
 * emf_advance runs the whole step.  The reference's own step order
 * (em1d/simulation.c:45-56, mods/em1d_param_scan/main.c) therefore gives the
 * same result, and other orders are not supported.
 *
 * Like the reference, the library keeps process-global state (the random
 * generator, the registry of simulations behind the structs): one thread
 * drives it.  Several simulations may live at once; for scans of many runs
 * on one GPU, the C-ABI's zc1_step_async is the faster route. */
#ifndef ZPIC_EM1D_SIMULATION_H
#define ZPIC_EM1D_SIMULATION_H
#include <stdint.h>
#include "particles.h"
#include "emf.h"
#include "current.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct Simulation {
    float dt;
    float tmax;
    int ndump;
    int n_species;
    t_species *species;
    t_emf emf;
    t_current current;
    int moving_window;
} t_simulation;

/* defined by the deck */
void sim_init(t_simulation *sim);
void sim_report(t_simulation *sim);

void sim_iter(t_simulation *sim);
void sim_report_energy(t_simulation *sim);
void sim_new(t_simulation *sim, int nx, float box, float dt, float tmax, int ndump, t_species *species,
             int n_species);
void sim_timings(t_simulation *sim, uint64_t t0, uint64_t t1);
void sim_add_laser(t_simulation *sim, t_emf_laser *laser);
void sim_delete(t_simulation *sim);
void sim_set_moving_window(t_simulation *sim);
void sim_set_smooth(t_simulation *sim, t_smooth *smooth);
void sim_set_ext_fld(t_simulation *sim, t_emf_ext_fld *ext_fld);
int report(int n, int ndump);

#ifdef __cplusplus
}
#endif
#endif
