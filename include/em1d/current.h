/* current.h -- electric current of the em1d drop-in API.  Layout as the
 * reference's em1d/current.h: a float3 buffer of nx + 3 cells (one lower,
 * two upper guard cells), J pointing at cell 0.  J_buf is a host mirror of
 * the filtered current of the last step, refreshed by current_report. */
#ifndef ZPIC_EM1D_CURRENT_H
#define ZPIC_EM1D_CURRENT_H
#include "zpic.h"
#ifdef __cplusplus
extern "C" {
#endif

enum smooth_type { NONE, BINOMIAL, COMPENSATED };

enum current_boundary { CURRENT_BC_NONE, CURRENT_BC_PERIODIC };

typedef struct Smooth {
    enum smooth_type xtype;
    int xlevel;
} t_smooth;

typedef struct Current {
    float3 *J;
    float3 *J_buf;
    int nx;
    int gc[2];
    float box;
    float dx;
    t_smooth smooth;
    float dt;
    int iter;
    enum current_boundary bc_type;
} t_current;

void current_new(t_current *current, int nx, float box, float dt);
void current_delete(t_current *current);
/* the phase calls of em1d/current.h:93-100: zeroing and the guard fold /
 * filter run inside the GPU step (see emf_advance) */
void current_zero(t_current *current);
void current_update(t_current *current);
void current_report(const t_current *current, const int jc);

#ifdef __cplusplus
}
#endif
#endif
