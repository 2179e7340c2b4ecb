/* current.h -- electric current density of the em2d drop-in API.
 * Struct layout as the reference's em2d/current.h:19-70.  J_buf is a host
 * mirror of the device current: it is refreshed by the reporting calls and
 * by sim_sync_host(). */
#ifndef ZPIC_EM2D_CURRENT_H
#define ZPIC_EM2D_CURRENT_H
#include "zpic.h"
#ifdef __cplusplus
extern "C" {
#endif

enum smooth_type { NONE, BINOMIAL, COMPENSATED };

typedef struct Smooth {
    enum smooth_type xtype;
    enum smooth_type ytype;
    int xlevel;
    int ylevel;
} t_smooth;

typedef struct Current {
    float3 *J;        /* cell (0,0) of J_buf */
    float3 *J_buf;    /* (nx+3)*(ny+3) cells, guard cells 1 below and 2 above */
    int nx[2];
    int nrow;
    int gc[2][2];
    float box[2];
    float dx[2];
    t_smooth smooth;
    float dt;
    int iter;
    int moving_window;
} t_current;

void current_new(t_current *current, int nx[], float box[], float dt);
void current_delete(t_current *current);
void current_zero(t_current *current);
void current_update(t_current *current);
void current_report(const t_current *current, const int jc);

#ifdef __cplusplus
}
#endif
#endif
