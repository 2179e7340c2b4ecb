/* emf.h -- EM fields of the em1d drop-in API.  Struct layouts as the
 * reference's em1d/emf.h: float3 buffers of nx + 3 cells (one lower, two
 * upper guard cells), E and B pointing at cell 0.  E_buf and B_buf are host
 * mirrors: they hold what the deck sets up (initial fields, lasers) until
 * the first step hands them to the GPU, and the device fields after each
 * report or emf_get_energy.  External fields are not supported by the 1-D
 * GPU step (emf_set_ext_fld stops the program, as the reference does for
 * invalid settings). */
#ifndef ZPIC_EM1D_EMF_H
#define ZPIC_EM1D_EMF_H
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
    float3 (*E_custom)(int, float, void *);
    float3 (*B_custom)(int, float, void *);
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
    float3 (*E_custom)(int, float, void *);
    float3 (*B_custom)(int, float, void *);
    void *E_custom_data;
    void *B_custom_data;
} t_emf_init_fld;

enum emf_diag { EFLD, BFLD, EPART, BPART };

enum emf_boundary { EMF_BC_NONE, EMF_BC_PERIODIC, EMF_BC_OPEN };

typedef struct EMF {
    float3 *E;
    float3 *B;
    float3 *E_buf;
    float3 *B_buf;
    float3 *E_part;
    float3 *B_part;
    int nx;
    int gc[2];
    float box;
    float dx;
    float dt;
    int iter;
    int moving_window;
    int n_move;
    enum emf_boundary bc_type;
    float3 mur_fld[2];
    float3 mur_tmp[2];
    t_emf_ext_fld ext_fld;
} t_emf;

typedef struct EMF_Laser {
    float start;
    float fwhm;
    float rise;
    float flat;
    float fall;
    float a0;
    float omega0;
    float polarization;
} t_emf_laser;

void emf_get_energy(const t_emf *emf, double energy[]);
void emf_new(t_emf *emf, int nx, float box, const float dt);
void emf_delete(t_emf *emf);
void emf_report(const t_emf *emf, const char field, const int fc);
void emf_add_laser(t_emf *const emf, t_emf_laser *laser);
void emf_init_fld(t_emf *const emf, t_emf_init_fld *init_fld);
void emf_set_ext_fld(t_emf *const emf, t_emf_ext_fld *ext_fld);
/* the last phase of sim_iter: here it runs the whole step of the simulation
 * that owns `emf` on the GPU (see simulation.h) */
void emf_advance(t_emf *emf, const t_current *current);
double emf_time(void);

#ifdef __cplusplus
}
#endif
#endif
