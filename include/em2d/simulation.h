/* simulation.h -- the em2d drop-in API: ZPIC's em2d C interface
 * (reference em2d/simulation.h:13-65) backed by libzpic_cuda.
 *
 * Link input decks against libzpic_em2d.so (which loads libzpic_cuda.so).
 * The time step runs on the GPU; t_species.part, t_emf.E_buf/B_buf and
 * t_current.J_buf are host mirrors in the reference layout.  By default
 * sim_iter keeps them valid as the reference's own buffers are: edits made
 * to the particle and field mirrors between steps are uploaded before the
 * step, and every mirror is refreshed after it (particles in the GPU's tile
 * order).  With ZPIC_EM2D_MIRRORS=demand in the environment at sim_new, the
 * per-step copies are skipped: the reports refresh what they write, and a
 * program that reads or edits the mirrors directly calls sim_sync_host()
 * before reading and sim_sync_device() after editing (two additions to the
 * reference API).  The per-phase calls (spec_advance, current_update,
 * emf_advance) never refresh the mirrors. */
#ifndef ZPIC_EM2D_SIMULATION_H
#define ZPIC_EM2D_SIMULATION_H
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

/* provided by the input deck */
void sim_init(t_simulation *sim);
void sim_report(t_simulation *sim);

void sim_iter(t_simulation *sim);
void sim_report_energy(t_simulation *sim);
void sim_new(t_simulation *sim, int nx[], float box[], float dt, float tmax, int ndump, t_species *species,
             int n_species);
int report(int n, int ndump);
void sim_timings(t_simulation *sim, uint64_t t0, uint64_t t1);
void sim_add_laser(t_simulation *sim, t_emf_laser *laser);
void sim_delete(t_simulation *sim);
void sim_set_moving_window(t_simulation *sim);
void sim_set_smooth(t_simulation *sim, t_smooth *smooth);
void sim_set_ext_fld(t_simulation *sim, t_emf_ext_fld *ext_fld);

/* additions: host mirrors <-> GPU state */
void sim_sync_host(t_simulation *sim);
void sim_sync_device(t_simulation *sim);
/* mirror policy of this simulation: 1 kept valid across every sim_iter (the
 * default), 0 refreshed on demand only (as ZPIC_EM2D_MIRRORS=demand) */
void sim_set_mirrors(t_simulation *sim, int every_step);
/* the libzpic_cuda handle behind a simulation (NULL if sim_new did not
 * create it), for callers that use both APIs on one run */
struct zc_sim *sim_gpu_handle(t_simulation *sim);
/* grid forms of emf_set_ext_fld / emf_init_fld: custom fields given as host
 * grids in the reference layout (every buffer cell), for callers whose
 * callbacks cannot return a float3 by value; types as enum emf_fld_type */
void emf_set_ext_fld_grid(t_emf *const emf, int E_type, const float E0[3], const float *E_grid, int B_type,
                          const float B0[3], const float *B_grid);
void emf_init_fld_grid(t_emf *const emf, const float *E_grid, const float *B_grid);
/* selects the GPU, the particle tile and the push build before sim_new
 * (defaults: device 0, 16 x 16 tiles, exact push) */
void sim_set_gpu_options(int device, int tile_x, int tile_y, int fast_math);

#ifdef __cplusplus
}
#endif
#endif
