/* emf.h -- electromagnetic fields of the em2d drop-in API.
 * Struct layouts as the reference's em2d/emf.h:20-157.  E_buf / B_buf are
 * host mirrors of the device fields, refreshed by the reporting calls and by
 * sim_sync_host(). */
#ifndef ZPIC_EM2D_EMF_H
#define ZPIC_EM2D_EMF_H
#include "zpic.h"
#include "current.h"
#ifdef __cplusplus
extern "C" {
#endif

enum emf_fld_type { EMF_FLD_TYPE_NONE, EMF_FLD_TYPE_UNIFORM, EMF_FLD_TYPE_CUSTOM };

typedef struct EMF_ExternalField {
    enum emf_fld_type E_type;
    enum emf_fld_type B_type;
    float3 E_0;
    float3 B_0;
    float3 (*E_custom)(int, float, int, float, void *);
    float3 (*B_custom)(int, float, int, float, void *);
    void *E_custom_data;
    void *B_custom_data;
    float3 *E_part_buf;
    float3 *B_part_buf;
} t_emf_ext_fld;

typedef struct EMF_InitialField {
    enum emf_fld_type E_type;
    enum emf_fld_type B_type;
    float3 E_0;
    float3 B_0;
    float3 (*E_custom)(int, float, int, float, void *);
    float3 (*B_custom)(int, float, int, float, void *);
    void *E_custom_data;
    void *B_custom_data;
} t_emf_init_fld;

enum emf_diag { EFLD, BFLD, EPART, BPART };

typedef struct EMF {
    float3 *E;
    float3 *B;
    float3 *E_buf;
    float3 *B_buf;
    float3 *E_part;
    float3 *B_part;
    int nx[2];
    int nrow;
    int gc[2][2];
    float box[2];
    float dx[2];
    float dt;
    int iter;
    int moving_window;
    int n_move;
    t_emf_ext_fld ext_fld;
} t_emf;

enum emf_laser_type { PLANE, GAUSSIAN };

typedef struct EMF_Laser {
    enum emf_laser_type type;
    float start;
    float fwhm;
    float rise;
    float flat;
    float fall;
    float a0;
    float omega0;
    float polarization;
    float W0;
    float focus;
    float axis;
} t_emf_laser;

void emf_get_energy(const t_emf *emf, double energy[]);
void emf_new(t_emf *emf, int nx[], float box[], const float dt);
void emf_delete(t_emf *emf);
void emf_report(const t_emf *emf, const char field, const int fc);
void emf_add_laser(t_emf *const emf, t_emf_laser *laser);
void emf_init_fld(t_emf *const emf, t_emf_init_fld *init_fld);
void emf_set_ext_fld(t_emf *const emf, t_emf_ext_fld *ext_fld);
void emf_advance(t_emf *emf, const t_current *current);
double emf_time(void);

#ifdef __cplusplus
}
#endif
#endif
