/* particles.h -- particle species of the em1d drop-in API.  Struct layouts
 * as the reference's em1d/particles.h.  `part` is a host mirror in the
 * reference record layout: spec_new loads it exactly as the reference does
 * (same generator, same order), the first step hands it to the GPU, and the
 * particle-based reports (and spec_sync_host) refresh it afterwards. */
#ifndef ZPIC_EM1D_PARTICLES_H
#define ZPIC_EM1D_PARTICLES_H
#include <stdint.h>
#include "zpic.h"
#include "emf.h"
#include "current.h"
#ifdef __cplusplus
extern "C" {
#endif

#define MAX_SPNAME_LEN 32

typedef struct Particle {
    int ix;
    float x;
    float ux;
    float uy;
    float uz;
} t_part;

enum density_type { UNIFORM, EMPTY, STEP, SLAB, RAMP, CUSTOM };

typedef struct Density {
    float n;
    enum density_type type;
    float start;
    float end;
    float ramp[2];
    float (*custom)(float, void *);
    void *custom_data;
    unsigned long total_np_inj;
    double custom_q_inj;
} t_density;

enum part_boundary { PART_BC_NONE, PART_BC_PERIODIC, PART_BC_OPEN };

typedef struct Species {
    char name[MAX_SPNAME_LEN + 1];
    t_part *part;
    int np;
    int np_max;
    float m_q;
    double energy;
    float q;
    int ppc;
    t_density density;
    float ufl[3];
    float uth[3];
    int nx;
    float dx;
    float box;
    float dt;
    int iter;
    int moving_window;
    int n_move;
    enum part_boundary bc_type;
    int n_sort;
} t_species;

void spec_new(t_species *spec, char name[], const float m_q, const int ppc, const float ufl[], const float uth[],
              const int nx, float box, const float dt, t_density *density);
void spec_delete(t_species *spec);
void spec_grow_buffer(t_species *spec, const int size);
/* a phase of sim_iter: the push of every species runs inside the GPU step
 * (see emf_advance) */
void spec_advance(t_species *spec, t_emf *emf, t_current *current);
uint64_t spec_npush(void);
double spec_time(void);
double spec_perf(void);

#define CHARGE 0x1000
#define PHA 0x2000
#define PARTICLES 0x3000
#define X1 0x0001
#define U1 0x0004
#define U2 0x0005
#define U3 0x0006
#define PHASESPACE(a, b) ((a) + (b)*16 + PHA)

void spec_deposit_pha(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2],
                      float *buf);
void spec_deposit_charge(const t_species *spec, float *charge);
void spec_report(const t_species *spec, const int rep_type, const int pha_nx[], const float pha_range[][2]);

/* addition: refreshes the host mirror (part, np, iter, n_move, energy) from
 * the GPU (no counterpart in the reference, whose buffers are the state) */
void spec_sync_host(t_species *spec);

#ifdef __cplusplus
}
#endif
#endif
