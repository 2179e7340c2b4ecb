/* zpic.h -- shared vector type and constants of the em1d drop-in API
 * (em1d/zpic.h). */
#ifndef ZPIC_EM1D_ZPIC_H
#define ZPIC_EM1D_ZPIC_H

typedef struct Float3 {
    float x;
    float y;
    float z;
} float3;

#ifndef M_PI
#define M_PI 3.14159265358979323846264338327950288
#endif
#ifndef M_PI_2
#define M_PI_2 1.57079632679489661923132169163975144
#endif
#ifndef M_PI_4
#define M_PI_4 0.785398163397448309615660845819875721
#endif

#endif
